"""CPU oracle pinned against the reference's own known-answer and property
tests (kinds 1-5 of unit_test/bundle_adjustment) and an independent scipy
projection."""
import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

from helpers import ALL_FIX_MASKS, abs_rel_ok, fixture_cases, full_scene, is_approx, single_key_scene

MASKS = {
    "normalized": 0,
    "radial": abi.COMPUTE_RADIAL,
    "decentering": abi.COMPUTE_DECENTERING,
    "intrinsic": abi.COMPUTE_RADIAL | abi.COMPUTE_DECENTERING | abi.COMPUTE_INTRINSIC,
}


def _dense_blocks(pb, ib, cb):
    return np.concatenate([pb[0], ib[0], cb[0]], axis=1)


@pytest.mark.parametrize("which", list(MASKS))
def test_reference_derivative_fixture(which):
    """test_camera_shared_analytical_derivative.cpp:746-770: analytical vs
    FFD(1e-6, 1e-8) isApprox 1e-5 on the fixed point/pose/intrinsics."""
    case = fixture_cases()[0]
    assert case["name"] == "reference_fixture"
    s, x = single_key_scene(case, MASKS[which])
    a = _dense_blocks(*oracle.jacobian(s, x))
    f = _dense_blocks(*oracle.jacobian(s, x, ffd=(1e-6, 1e-8)))
    assert is_approx(f, a, 1e-5), np.abs(f - a).max()


@pytest.mark.parametrize("case_index", range(17))
def test_projection_matches_independent_golden(case_index):
    case = fixture_cases()[case_index]
    s, x = single_key_scene(case, MASKS["intrinsic"])
    y = oracle.vector_function(s, x)
    np.testing.assert_allclose(y, case["key"], rtol=1e-12, atol=1e-9)
    s0, x0 = single_key_scene(case, 0)
    np.testing.assert_allclose(oracle.vector_function(s0, x0), case["normalized"], rtol=1e-12,
                               atol=1e-12)


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
def test_jacobian_vs_ffd_all_fix_masks(fix_mask):
    """test_camera_shared_jacobian_matrix_calculator.cpp:121,465-491."""
    s = full_scene(fix_mask)
    a = oracle.jacobian(s, s.x0)
    f = oracle.jacobian(s, s.x0, ffd=(1e-6, 1e-8))
    for blk_a, blk_f, fixed in zip(a, f, [fix_mask & 1, fix_mask & 2, fix_mask & 4]):
        if fixed:
            continue
        ok, e, r = abs_rel_ok(blk_f, blk_a, 1e-3)
        assert ok, (e, r)


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
def test_vector_function_vs_generator(fix_mask):
    """test_camera_shared_vector_function.cpp:163-194: f(x_true) reproduces
    the generator's keys (noise-free) to 1e-8."""
    s = full_scene(fix_mask)
    y = oracle.vector_function(s, s.x_true)
    keys, _ = synthetic.project(s.points[s.feature_maps[:, 1]], s.images[s.feature_maps[:, 0]],
                                s.cameras[s.image_camera_map[s.feature_maps[:, 0]]], s.intrinsic_mask)
    assert is_approx(y[:2 * s.number_of_keys], keys.reshape(-1), 1e-8)
    rows = abi.constraint_rows(s)
    np.testing.assert_array_equal(y[2 * s.number_of_keys:], s.x_true[[r[0] for r in rows]])


def _dense_lambda(s):
    K = s.number_of_keys
    rows = abi.constraint_rows(s)
    L = np.zeros((2 * K + len(rows),) * 2)
    kci = s.key_covariance_inverse if s.key_covariance_inverse is not None else \
        np.tile(np.eye(2), (K, 1, 1))
    for k in range(K):
        L[2 * k:2 * k + 2, 2 * k:2 * k + 2] = kci[k]
    w = s.constraint_weights if s.constraint_weights is not None else np.ones(len(rows))
    for c in range(len(rows)):
        L[2 * K + c, 2 * K + c] = w[c]
    return L


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
def test_builder_vs_dense(fix_mask):
    """test_camera_shared_normal_equation_builder.hpp:505-601: block N and g
    vs dense J^T Lambda J and J^T Lambda r (r = f(x) - y) at 1e-8."""
    s = full_scene(fix_mask)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    J = oracle.dense_jacobian(s, s.x0)
    L = _dense_lambda(s)
    r = oracle.vector_function(s, s.x0) - s.near_y
    Nd = J.T @ L @ J
    gd = J.T @ L @ r
    ok, e, rel = abs_rel_ok(Nd, N, 1e-8)
    assert ok, (e, rel)
    ok, e, rel = abs_rel_ok(gd, g, 1e-8)
    assert ok, (e, rel)


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
@pytest.mark.parametrize("faithful", [True, False])
def test_schur_solver_property(fix_mask, faithful):
    """test_camera_shared_normal_equation_solver.hpp:259-325: with mu = max
    diag(N), (N + mu I) delta = g elementwise at 1e-5 abs & rel."""
    s = full_scene(fix_mask)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    mu = float(np.max(np.diag(N)))
    err, dx = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=faithful)
    assert err == 0
    lhs = (N + mu * np.eye(len(g))) @ dx
    ok, e, rel = abs_rel_ok(g, lhs, 1e-5)
    assert ok, (e, rel)


def test_schur_small_mu_matches_dense_solve():
    s = full_scene(abi.FIX_CAMERAS, constraints=False)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    mu = 1e-3 * float(np.max(np.diag(N)))
    err, dx = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=True)
    assert err == 0
    ref = np.linalg.solve(N + mu * np.eye(len(g)), g)
    np.testing.assert_allclose(dx, ref, rtol=1e-7, atol=1e-9 * np.abs(ref).max())


def test_lm_config0_converges_and_modes_agree():
    s = synthetic.config(0)
    opt = abi.make_options(max_iterations=20)
    err, x_fast, rep = oracle.lm_solve(s, options=opt, faithful=False)
    assert err == 0
    err, x_faith, rep2 = oracle.lm_solve(s, options=opt, faithful=True)
    assert err == 0
    assert rep.final_cost < 1e-2 * rep.initial_cost
    # noise is N(0,1) px per coordinate: the optimum RMSE is close to sqrt(2)*sqrt((2K-dof)/2K)
    assert 1.0 < rep.final_rmse < 1.3
    assert abs(rep.final_cost - rep2.final_cost) <= 1e-9 * rep.final_cost
    np.testing.assert_allclose(x_fast, x_faith, atol=1e-8)
    assert rep.final_cost < oracle.cost(s, s.x_true, s.near_y)


def test_lm_end_to_end_accuracy_like_reference():
    """test_camera_shared_levenberg_marquardt_optimizor.cpp:186-212: the
    mean key residual after optimisation is within 2 sigma."""
    s = synthetic.ring_scene(num_images=8, num_points=400, obs_per_point=4, seed=5)
    err, x, rep = oracle.lm_solve(s, options=abi.make_options(max_iterations=50))
    assert err == 0
    y = oracle.vector_function(s, x)
    res = np.linalg.norm((y - s.near_y).reshape(-1, 2), axis=1)
    assert res.mean() <= 2.0 * np.sqrt(2.0)


def test_invalid_inputs_rejected():
    s = synthetic.ring_scene(num_images=4, num_points=20, obs_per_point=2, seed=1)
    bad = synthetic.ring_scene(num_images=4, num_points=20, obs_per_point=2, seed=1)
    bad.feature_maps = bad.feature_maps.copy()
    bad.feature_maps[3, 0] = 99
    with pytest.raises(RuntimeError):
        oracle.cost(bad, bad.x0, bad.near_y)
    dup = synthetic.ring_scene(num_images=4, num_points=20, obs_per_point=2, seed=1)
    dup.feature_maps = dup.feature_maps.copy()
    dup.feature_maps[1] = dup.feature_maps[0]
    with pytest.raises(RuntimeError):
        oracle.cost(dup, dup.x0, dup.near_y)
    assert oracle.cost(s, s.x0, s.near_y) > 0


def test_huber_cost_and_weights():
    s = synthetic.ring_scene(num_images=6, num_points=100, obs_per_point=3, seed=2)
    r = (oracle.vector_function(s, s.x0) - s.near_y).reshape(-1, 2)
    sq = (r ** 2).sum(1)
    rho = np.where(sq <= 1.0, sq, 2 * np.sqrt(sq) - 1.0)
    c = oracle.cost(s, s.x0, s.near_y, loss=abi.LOSS_HUBER, huber_delta=1.0)
    np.testing.assert_allclose(c, rho.sum(), rtol=1e-12)


def _dense_lambda_with_priors(s):
    """The dense inverse covariance of y: key blocks, then 3x3 prior blocks
    (ba_gcp_constrained_y_covariance_inverse.hpp:18-25)."""
    K = s.number_of_keys
    n = abi.y_size(s)
    L = np.zeros((n, n))
    for k in range(K):
        L[2 * k:2 * k + 2, 2 * k:2 * k + 2] = s.key_covariance_inverse[k]
    b = 2 * K + len(abi.constraint_rows(s))
    for i in range(len(s.point_priors)):
        L[b + 3 * i:b + 3 * i + 3, b + 3 * i:b + 3 * i + 3] = s.prior_information[i]
    return L


def test_gcp_builder_vs_dense():
    """test_ba_gcp_constrained_normal_equation_builder.cpp:150-190: the block
    normal equations with the ground control points' 3x3 priors against
    dense J^T Lambda J and J^T Lambda r at 1e-8."""
    s = synthetic.gcp_scene(seed=1, num_images=6, num_points=80, num_gcps=5)
    assert abi.y_size(s) == len(s.near_y) == 2 * s.number_of_keys + 15
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    J = oracle.dense_jacobian(s, s.x0)
    L = _dense_lambda_with_priors(s)
    r = oracle.vector_function(s, s.x0) - s.near_y
    ok, e, rel = abs_rel_ok(J.T @ L @ J, N, 1e-8)
    assert ok, (e, rel)
    ok, e, rel = abs_rel_ok(J.T @ L @ r, g, 1e-8)
    assert ok, (e, rel)
    # the prior rows of y are copies of the prior points (ba_gcp_constrained_vector_function.hpp:100-108)
    y = oracle.vector_function(s, s.x0)
    P = np.asarray(s.x0[:3 * s.number_of_points]).reshape(-1, 3)
    np.testing.assert_array_equal(y[2 * s.number_of_keys:].reshape(-1, 3), P[s.point_priors])
    c = oracle.cost(s, s.x0, s.near_y)
    assert abs(c - r @ L @ r) <= 1e-10 * c


def test_gcp_priors_fix_the_gauge():
    """test_ba_gcp_constrained_gauge.cpp: with ground control points the
    solution lands in the points' own frame, off the truth by no more than
    the control points' own noise, and fits the data better than the truth."""
    s = synthetic.gcp_scene(seed=2, num_images=8, num_points=200, num_gcps=6)
    err, x, rep = oracle.lm_solve(s, options=abi.make_options(max_iterations=30))
    assert err == 0 and rep.stop_reason == abi.STOP_SMALL_STEP
    assert rep.final_cost < oracle.cost(s, s.x_true, s.near_y)
    P = x[:3 * s.number_of_points].reshape(-1, 3)
    e = np.sqrt(np.mean(np.sum((P - s.points) ** 2, axis=1)))
    gy = s.near_y[2 * s.number_of_keys:].reshape(-1, 3)
    e_gcp = np.sqrt(np.mean(np.sum((gy - s.points[s.point_priors]) ** 2, axis=1)))
    assert e < 1.5 * e_gcp, (e, e_gcp)


def test_prior_bad_index_rejected():
    s = synthetic.gcp_scene(seed=1, num_images=6, num_points=80, num_gcps=3)
    s.point_priors = [0, 1, s.number_of_points]
    with pytest.raises(RuntimeError):
        oracle.cost(s, s.x0, s.near_y)


def test_triangulation_oracle_noise_free_and_refines():
    """Multi-view triangulation restatement: exact on noise-free tracks with
    distortion (DLT of undistorted keys, then LM), and the LM lowers the
    reprojection cost of the DLT start."""
    b = synthetic.triangulation_batch(seed=1, num_points=500, noise=0.0)
    P, st = oracle.triangulate(b)
    assert np.all(st == 0) and np.max(np.abs(P - b.points)) < 1e-9
    b = synthetic.triangulation_batch(seed=2, num_points=500, noise=1.0)
    P0, _ = oracle.triangulate(b, abi.make_options(max_iterations=0))
    P1, _ = oracle.triangulate(b)
    k = np.diff(b.track_offsets)

    def cost(Pts):
        r = synthetic.project_views(b.intrinsics, b.extrinsics, b.track_views,
                                    np.repeat(Pts, k, axis=0)) - b.track_keys
        return float(np.sum(r * r))

    assert cost(P1) < cost(P0)
