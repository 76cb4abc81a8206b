/*
 * gba_oracle.h -- CPU FP64 oracle for the bundle-adjustment path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain C++ restatement of the
 * reference's camera-shared bundle-adjustment path (hs_sfm,
 * include/hs_sfm/bundle_adjustment/camera_shared_*), used by the tests as the
 * checker and by the benchmark as the timed CPU baseline.  The product
 * (libgba.so) never links, loads or calls it.
 *
 * Parity pins (see tests/test_oracle_*.py):
 *  - the reference's known-answer derivative fixture
 *    (unit_test/bundle_adjustment/test_camera_shared_analytical_derivative.cpp:746-770),
 *    analytical vs forward-finite-difference Jacobian at 1e-5;
 *  - Jacobian vs FFD over the seven fix masks at 1e-3 abs & rel
 *    (test_camera_shared_jacobian_matrix_calculator.cpp:121,465-491);
 *  - block normal equations vs dense J^T Lambda J, J^T Lambda r at 1e-8
 *    (test_camera_shared_normal_equation_builder.hpp:505-601);
 *  - Schur solve property (N + mu I) delta = g at 1e-5
 *    (test_camera_shared_normal_equation_solver.hpp:293-325);
 *  - projection against an independent scipy Rodrigues implementation
 *    (tests/golden/make_golden.py).
 * The LM driver lives in an absent dependency (hs_optimizor @746e478); its
 * restatement follows Madsen, Nielsen & Tingleff (2004) Alg. 3.16 and its
 * trajectory parity with the reference is unpinned.
 */
#ifndef GBA_ORACLE_H_
#define GBA_ORACLE_H_

#include "../include/gba.h"

#ifdef __cplusplus
extern "C" {
#endif

int oracle_vector_function(const gba_problem* problem, const double* x,
                           double* y);

/* Analytical Jacobian blocks per key (row-major 2x3, 2x6, 2xc). */
int oracle_jacobian(const gba_problem* problem, const double* x,
                    double* point_blocks, double* image_blocks,
                    double* camera_blocks);

/* Forward-finite-difference Jacobian blocks per key
 * (camera_shared_forward_finite_difference_jacobian_matrix_calculator.hpp:51-241). */
int oracle_ffd_jacobian(const gba_problem* problem, const double* x,
                        double delta, double min_delta, double* point_blocks,
                        double* image_blocks, double* camera_blocks);

/* Dense y_size x x_size Jacobian including constraint rows (row-major). */
int oracle_dense_jacobian(const gba_problem* problem, const double* x,
                          double* jacobian);

/* Block normal equations at x, written out densely: N [x_size^2] row-major
 * and g [x_size], residual r = f(x) - near_y. */
int oracle_normal_equation_dense(const gba_problem* problem, const double* x,
                                 const double* near_y, double* normal,
                                 double* gradient);

/* Sum of r^T Lambda r (loss: GBA_LOSS_*). */
int oracle_cost(const gba_problem* problem, const double* x,
                const double* near_y, int32_t loss, double huber_delta,
                double* cost);

/* Solve (N + mu I) delta = g.  faithful=1 keeps the reference's loop order
 * (O(I^2 P) sparse lookups), faithful=0 accumulates point-major. */
int oracle_schur_step(const gba_problem* problem, const double* x,
                      const double* near_y, double mu, int32_t faithful,
                      int32_t loss, double huber_delta, double* delta_x);

/* Full LM solve (MNT Alg. 3.16 as bound by the reference's traits). */
int oracle_lm_solve(const gba_problem* problem, const double* near_y,
                    const gba_options* options, int32_t faithful,
                    double* x_inout, gba_report* report);

/* Times one LM iteration (linearize + reduced system + factor + back-sub +
 * candidate cost) of the faithful restatement at x.  The O(I^2 P)
 * reduced-system loop is run over every row_stride-th weighted image only
 * and its time is scaled by row_stride; the factorization runs on the full
 * reduced system.  seconds[0] = estimated full iteration, seconds[1..5] =
 * linearize, reduced system (scaled), factor, back-substitution, cost. */
int oracle_time_faithful_iteration(const gba_problem* problem,
                                   const double* near_y, const double* x,
                                   double mu, int32_t row_stride,
                                   double* seconds);

/* Batched multi-view triangulation (gba_oracle_triangulate.cpp): DLT of the
 * undistorted keys, then LM on each point (triangulate/multiple_view_*). */
int oracle_triangulate(const gba_triangulation* problem, const gba_options* options,
                       double* points, int32_t* point_status);

#ifdef __cplusplus
}
#endif

#endif
