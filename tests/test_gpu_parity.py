"""GPU parity: every stage of libgba.so against the CPU FP64 oracle, through
the C ABI.  Tolerances: FP64 path to 1e-9 relative or tighter per stage;
the mixed FP32/FP64 path by the acceptance rule of the final results --
final cost within 1e-6 relative and reprojection RMSE within 1e-4 px of the
FP64 oracle."""
import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6
RMSE_ATOL = 1e-4


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def distorted_ring(seed=11, num_images=8, num_points=300, k=4, decentering=True):
    mask = abi.COMPUTE_RADIAL | abi.COMPUTE_INTRINSIC | (abi.COMPUTE_DECENTERING if decentering else 0)
    s = synthetic.ring_scene(num_images=num_images, num_points=num_points, obs_per_point=k,
                             seed=seed, mask=mask, fix_mask=abi.FIX_CAMERAS)
    rng = np.random.default_rng(seed)
    cam = s.cameras.copy()
    cam[0, 0:2] = rng.uniform(-0.05, 0.05, 2)
    if decentering:
        cam[0, 3:5] = rng.uniform(-1e-3, 1e-3, 2)
    s.cameras = cam
    keys, _ = synthetic.project(s.points[s.feature_maps[:, 1]], s.images[s.feature_maps[:, 0]],
                                cam[s.image_camera_map[s.feature_maps[:, 0]]], mask)
    s.near_y = (keys + rng.normal(0, 1.0, keys.shape)).reshape(-1)
    return s


def shuffled(s, seed=0):
    """The same problem with its keys in a random order."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(s.number_of_keys)
    t = synthetic.Scene(**{**s.__dict__})
    t.feature_maps = s.feature_maps[perm]
    t.near_y = s.near_y.reshape(-1, 2)[perm].reshape(-1)
    if s.key_covariance_inverse is not None:
        t.key_covariance_inverse = s.key_covariance_inverse[perm]
    return t


# ---------------------------------------------------------------- stages
@pytest.mark.parametrize("maker", ["cfg0", "distorted"])
def test_vector_function_fp64(gba, maker):
    s = synthetic.config(0) if maker == "cfg0" else shuffled(distorted_ring())
    y_gpu = gba.vector_function(s, s.x0)
    y_ref = oracle.vector_function(s, s.x0)
    np.testing.assert_allclose(y_gpu, y_ref, rtol=1e-13, atol=1e-10)


@pytest.mark.parametrize("precision,tol", [(abi.PRECISION_FP64, 1e-10), (abi.PRECISION_MIXED, 2e-4)])
def test_jacobian(gba, precision, tol):
    s = shuffled(distorted_ring())
    jp, ji = gba.jacobian(s, s.x0, precision)
    pb, ib, _ = oracle.jacobian(s, s.x0)
    for got, ref in ((jp, pb), (ji, ib)):
        scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
        assert np.max(np.abs(got - ref) / scale) < tol


def test_jacobian_near_zero_rotation(gba):
    """theta -> 0: the reference formula divides by zero; the device uses
    the series and must match the oracle evaluated just off zero."""
    s = synthetic.ring_scene(num_images=4, num_points=30, obs_per_point=2, seed=3)
    x = s.x0.copy()
    P = s.number_of_points
    x[3 * P:3 * P + 3] = [1e-7, -2e-7, 5e-8]   # image 0 nearly unrotated
    x[3 * P + 5] += 20.0                       # keep its points in front
    jp, ji = gba.jacobian(s, x)
    pb, ib, _ = oracle.jacobian(s, x)
    np.testing.assert_allclose(ji, ib, rtol=1e-6, atol=1e-6 * np.abs(ib).max())
    np.testing.assert_allclose(jp, pb, rtol=1e-6, atol=1e-6 * np.abs(pb).max())


@pytest.mark.parametrize("loss", [abi.LOSS_TRIVIAL, abi.LOSS_HUBER])
@pytest.mark.parametrize("weights", [False, True])
@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_cost(gba, loss, weights, precision):
    """FP64 path: FP64 projection, 1e-12.  Mixed path: double-float
    projection, whitening and squares (about 48 bits), FP64 block sums: 1e-12
    for inliers; Huber terms of outliers are formed in FP32 (1e-9)."""
    s = shuffled(distorted_ring())
    if weights:
        rng = np.random.default_rng(2)
        A = rng.normal(0, 0.3, size=(s.number_of_keys, 2, 2))
        s.key_covariance_inverse = np.linalg.inv(np.einsum('kij,klj->kil', A, A) + np.eye(2))
    opt = abi.make_options(loss=loss, huber_delta=1.0, precision=precision)
    c_gpu = gba.cost(s, s.x0, options=opt)
    c_ref = oracle.cost(s, s.x0, s.near_y, loss=loss, huber_delta=1.0)
    tol = 1e-12 if (precision == abi.PRECISION_FP64 or loss == abi.LOSS_TRIVIAL) else 1e-9
    assert abs(c_gpu - c_ref) <= tol * c_ref, (c_gpu, c_ref)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_schur_step(gba, precision):
    s = shuffled(distorted_ring(num_images=40, num_points=600, k=5), seed=1)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    for mu in (float(np.max(np.diag(N))), 1e-3 * float(np.max(np.diag(N)))):
        dx = gba.schur_step(s, s.x0, mu, options=abi.make_options(precision=precision))
        err, dref = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=False)
        assert err == 0
        rel = np.linalg.norm(dx - dref) / np.linalg.norm(dref)
        assert rel < (1e-9 if precision == abi.PRECISION_FP64 else 5e-3), rel
        if precision == abi.PRECISION_FP64:
            # the reference solver property (N + mu I) delta = g at 1e-5
            lhs = N @ dx + mu * dx
            err_abs = np.abs(lhs - g)
            err_rel = err_abs / np.maximum(np.abs(g), 1e-300)
            assert np.all((err_abs <= 1e-5) | (err_rel <= 1e-5))


# ---------------------------------------------------------------- solves
def _lm_opts(precision, iters=20):
    return abi.make_options(max_iterations=iters, eps1=0.0, eps2=0.0, precision=precision)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_lm_config0_matches_oracle(gba, precision):
    s = synthetic.config(0)
    x, rep = gba.solve(s, _lm_opts(precision))
    err, x_ref, rref = oracle.lm_solve(s, options=_lm_opts(abi.PRECISION_FP64))
    assert err == 0 and rep.status == 0
    assert rep.iterations == 20
    assert abs(rep.initial_cost - rref.initial_cost) <= 1e-12 * rref.initial_cost
    assert abs(rep.final_cost - rref.final_cost) <= COST_RTOL * rref.final_cost
    c_x = oracle.cost(s, x, s.near_y)   # the returned x, evaluated by the oracle
    assert abs(c_x - rref.final_cost) <= COST_RTOL * rref.final_cost
    rmse = np.sqrt(c_x / s.number_of_keys)
    assert abs(rmse - rref.final_rmse) <= RMSE_ATOL


def test_lm_with_stopping_criteria_fp64(gba):
    s = synthetic.config(0)
    opt = abi.make_options(max_iterations=50)
    x, rep = gba.solve(s, opt)
    err, x_ref, rref = oracle.lm_solve(s, options=opt)
    assert rep.stop_reason == rref.stop_reason
    assert rep.iterations == rref.iterations
    assert rep.accepted == rref.accepted
    np.testing.assert_allclose(x, x_ref, rtol=0, atol=1e-7)


def test_lm_function_tolerance_stop(gba):
    # Ceres' function_tolerance: stop after an accepted step that lowers the
    # cost by at most ftol of it (camera_shared_ceres_optimizor.hpp:478)
    s = synthetic.config(0)
    opt = abi.make_options(max_iterations=50, eps1=0.0, eps2=0.0, function_tolerance=1e-6)
    x, rep = gba.solve(s, opt)
    err, x_ref, rref = oracle.lm_solve(s, options=opt)
    assert rref.stop_reason == abi.STOP_SMALL_COST_CHANGE and rref.iterations < 50
    assert rep.stop_reason == rref.stop_reason
    assert rep.iterations == rref.iterations and rep.accepted == rref.accepted
    np.testing.assert_allclose(x, x_ref, rtol=0, atol=1e-7)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_lm_distorted_with_key_weights(gba, precision):
    s = shuffled(distorted_ring(num_images=12, num_points=500, k=5), seed=4)
    rng = np.random.default_rng(9)
    A = rng.normal(0, 0.2, size=(s.number_of_keys, 2, 2))
    s.key_covariance_inverse = np.linalg.inv(np.einsum('kij,klj->kil', A, A) + np.eye(2))
    x, rep = gba.solve(s, _lm_opts(precision, 15))
    err, x_ref, rref = oracle.lm_solve(s, options=_lm_opts(abi.PRECISION_FP64, 15))
    assert abs(rep.final_cost - rref.final_cost) <= COST_RTOL * rref.final_cost
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL   # plain, unweighted residuals


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_lm_huber_with_outliers(gba, precision):
    s = synthetic.ring_scene(num_images=10, num_points=800, obs_per_point=5, seed=21)
    rng = np.random.default_rng(21)
    y = s.near_y.reshape(-1, 2).copy()
    out = rng.random(len(y)) < 0.01
    y[out] = np.stack([rng.uniform(0, 1920, out.sum()), rng.uniform(0, 1080, out.sum())], 1)
    s.near_y = y.reshape(-1)
    opt = abi.make_options(max_iterations=20, eps1=0.0, eps2=0.0, precision=precision,
                           loss=abi.LOSS_HUBER, huber_delta=1.0)
    x, rep = gba.solve(s, opt)
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(
        max_iterations=20, eps1=0.0, eps2=0.0, loss=abi.LOSS_HUBER, huber_delta=1.0))
    assert abs(rep.final_cost - rref.final_cost) <= COST_RTOL * rref.final_cost
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL   # outliers included, no loss


def test_medium_grid_mixed_vs_fp64_oracle(gba):
    s = synthetic.grid_scene(num_images=48, num_points=6000, seed=5)
    opt = _lm_opts(abi.PRECISION_MIXED, 10)
    x, rep = gba.solve(s, opt)
    err, x_ref, rref = oracle.lm_solve(s, options=_lm_opts(abi.PRECISION_FP64, 10))
    assert abs(rep.final_cost - rref.final_cost) <= COST_RTOL * rref.final_cost
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL


# ---------------------------------------------------------------- batching
def test_batch_equals_alone_bitwise(gba):
    """Each window's result is the same alone and in the mix."""
    wins = synthetic.window_batch(num_windows=6, seed=7, points_range=(300, 1500))
    opt = _lm_opts(abi.PRECISION_MIXED, 10)
    xs, reps = gba.solve_batch(wins, opt)
    for w, xb, rb in zip(wins, xs, reps):
        xa, ra = gba.solve(w, opt)
        assert ra.final_cost == rb.final_cost
        np.testing.assert_array_equal(xa, xb)


def test_batch_windows_match_oracle(gba):
    wins = synthetic.window_batch(num_windows=8, seed=8, points_range=(300, 2000))
    for precision in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        xs, reps = gba.solve_batch(wins, _lm_opts(precision, 10))
        for w, r in zip(wins, reps):
            err, xr, rr = oracle.lm_solve(w, options=_lm_opts(abi.PRECISION_FP64, 10))
            assert abs(r.final_cost - rr.final_cost) <= COST_RTOL * rr.final_cost, (w.name, precision)


def test_plan_rerun_is_deterministic(gba):
    s = synthetic.ring_scene(num_images=20, num_points=3000, obs_per_point=5, seed=2)
    plan = gba.Plan([s], _lm_opts(abi.PRECISION_MIXED, 8))
    plan.run()
    plan.synchronize()
    x1 = plan.x(0)
    plan.run()
    plan.synchronize()
    x2 = plan.x(0)
    np.testing.assert_array_equal(x1, x2)
    assert plan.launches() > 0
    plan.close()


def test_profile_mode_matches_graph_mode(gba):
    s = synthetic.ring_scene(num_images=12, num_points=1000, obs_per_point=4, seed=6)
    a, ra = gba.solve(s, _lm_opts(abi.PRECISION_MIXED, 6))
    o = _lm_opts(abi.PRECISION_MIXED, 6)
    o.profile = 1
    b, rb = gba.solve(s, o)
    np.testing.assert_array_equal(a, b)
    assert sum(rb.stage_ms) > 0


# ---------------------------------------------------------------- errors
def test_errors_are_reported(gba):
    s = synthetic.ring_scene(num_images=4, num_points=20, obs_per_point=2, seed=1)
    bad = synthetic.Scene(**{**s.__dict__})
    bad.feature_maps = s.feature_maps.copy()
    bad.feature_maps[0, 0] = 17
    with pytest.raises(gba.GbaError) as e:
        gba.solve(bad)
    assert e.value.status == abi.GBA_ERR_BAD_INDEX
    dup = synthetic.Scene(**{**s.__dict__})
    dup.feature_maps = s.feature_maps.copy()
    dup.feature_maps[1] = dup.feature_maps[0]
    with pytest.raises(gba.GbaError) as e:
        gba.solve(dup)
    assert e.value.status == abi.GBA_ERR_DUPLICATE
    all_fixed = synthetic.Scene(**{**s.__dict__})
    all_fixed.fix_mask = abi.FIX_POINTS | abi.FIX_IMAGES | abi.FIX_CAMERAS
    with pytest.raises(gba.GbaError) as e:
        gba.solve(all_fixed, x0=np.zeros(0))
    assert e.value.status == abi.GBA_ERR_UNSUPPORTED


def test_nan_observation_reports_status(gba):
    s = synthetic.ring_scene(num_images=4, num_points=20, obs_per_point=2, seed=1)
    s.near_y = s.near_y.copy()
    s.near_y[5] = np.nan
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s)
    assert e.value.status == abi.GBA_ERR_NAN


def test_plan_batched_x_and_reports_equal_per_problem_calls(gba):
    # gba_plan_set_initial_x_all / gba_plan_get_all against the per-problem calls
    scenes = synthetic.window_batch(num_windows=6, seed=31, images_range=(5, 12),
                                    points_range=(200, 900))
    scenes.append(synthetic.full_model_scene(seed=32, num_images=8, num_points=300,
                                             obs_per_point=4))   # free cameras
    plan = gba.Plan(scenes, abi.make_options(max_iterations=5, eps1=0.0, eps2=0.0))
    xs0, reps0 = plan.get_all()            # before a run: x0
    for q, s in enumerate(scenes):
        np.testing.assert_array_equal(xs0[q], s.x0)
    plan.run()
    plan.synchronize()
    xs, reps = plan.get_all()
    for q in range(len(scenes)):
        np.testing.assert_array_equal(xs[q], plan.x(q))
        r = plan.report(q)
        assert (reps[q].final_cost, reps[q].iterations, reps[q].status) == \
            (r.final_cost, r.iterations, r.status)
    plan.close()


def test_concurrent_solves_from_host_threads(gba):
    # gba_solve is re-entrant: solves on several host threads at once (each
    # plan has its own stream; ctypes releases the GIL) give the same bits as
    # the same solves one after another
    import threading
    scenes = [synthetic.ring_scene(num_images=10 + 2 * i, num_points=1500, obs_per_point=5, seed=40 + i)
              for i in range(6)]
    opt = abi.make_options(max_iterations=10, eps1=0.0, eps2=0.0, precision=abi.PRECISION_MIXED)
    alone = [gba.solve(s, opt) for s in scenes]
    out = [None] * len(scenes)

    def work(i):
        out[i] = gba.solve(scenes[i], opt)

    threads = [threading.Thread(target=work, args=(i,)) for i in range(len(scenes))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for (x0, r0), (x1, r1) in zip(alone, out):
        assert np.array_equal(x0, x1) and r0.final_cost == r1.final_cost


def test_batch_create_submit_poll(gba):
    # the asynchronous batch face (gba_batch_*): submit returns before the
    # solve ends, poll answers BUSY until it has, then gives gba_solve_batch's bits
    import ctypes as C
    L = gba.lib()
    scenes = synthetic.window_batch(num_windows=5, seed=51, images_range=(5, 12),
                                    points_range=(300, 1200))
    opt = abi.make_options(max_iterations=8, eps1=0.0, eps2=0.0, precision=abi.PRECISION_MIXED)
    cps = [abi.CProblem(s) for s in scenes]
    arr = (abi.Problem * len(cps))(*[c.problem for c in cps])
    ys = [np.ascontiguousarray(s.near_y, dtype=np.float64) for s in scenes]
    yp = (C.POINTER(C.c_double) * len(ys))(*[abi.dptr(y) for y in ys])
    h = C.c_void_p()
    assert L.gba_batch_create(arr, yp, len(scenes), C.byref(opt), C.byref(h)) == abi.GBA_OK
    x0 = [np.ascontiguousarray(s.x0, dtype=np.float64) for s in scenes]
    x0p = (C.POINTER(C.c_double) * len(x0))(*[abi.dptr(x) for x in x0])
    xs = [np.zeros_like(x) for x in x0]
    xp = (C.POINTER(C.c_double) * len(xs))(*[abi.dptr(x) for x in xs])
    reps = (abi.Report * len(xs))()
    for _ in range(2):   # a batch can be submitted again
        assert L.gba_batch_submit(h, x0p) == abi.GBA_OK
        for _ in range(200000):
            st = L.gba_batch_poll(h, xp, reps)
            if st != abi.GBA_ERR_BUSY:
                break
        assert st == abi.GBA_OK
        ref_x, ref_r = gba.solve_batch(scenes, opt)
        for q in range(len(scenes)):
            np.testing.assert_array_equal(xs[q], ref_x[q])
            assert reps[q].final_cost == ref_r[q].final_cost
    assert L.gba_batch_destroy(h) == abi.GBA_OK


def test_folded_control_matches_control_kernels(gba, monkeypatch):
    """The LM step and accept decisions run in the last CTA of the
    back-substitution and of the candidate cost (no separate control
    launches); the same solve with the separate control kernels
    (GBA_CTRL_KERNELS=1) follows the same trajectory (the sums over chunk
    partials are taken by CTAs of another width, so the bits may differ)."""
    s = distorted_ring(seed=17, num_images=12, num_points=900, k=5)
    for precision in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        opt = _lm_opts(precision, 12)
        x1, r1 = gba.solve(s, opt)
        plan = gba.Plan([s], _lm_opts(precision, 12))
        plan.run()
        plan.synchronize()
        launches_folded = plan.launches()
        plan.close()
        monkeypatch.setenv("GBA_CTRL_KERNELS", "1")
        x2, r2 = gba.solve(s, opt)
        plan = gba.Plan([s], _lm_opts(precision, 12))
        plan.run()
        plan.synchronize()
        launches_kernels = plan.launches()
        plan.close()
        monkeypatch.delenv("GBA_CTRL_KERNELS")
        assert r1.status == r2.status == abi.GBA_OK
        assert (r1.accepted, r1.rejected, r1.iterations) == (r2.accepted, r2.rejected, r2.iterations)
        assert abs(r1.final_cost - r2.final_cost) <= 1e-10 * r2.final_cost
        np.testing.assert_allclose(x1, x2, rtol=1e-8, atol=1e-8)
        assert launches_folded == launches_kernels - 2 * 12
