"""The header-only C++ facade (include/gba/camera_shared.hpp): builds and
links against libgba.so, keeps the reference's Err for a size mismatch
(camera_shared_levenberg_marquardt_optimizor.hpp:48-51), and on a GPU
reaches the oracle's final cost."""
import os
import subprocess

import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

from facade_util import build_facade, write_gcp_problem, write_problem, write_triangulation


def test_facade_builds_and_rejects_bad_initial_x(tmp_path):
    exe = build_facade(str(tmp_path))
    s = synthetic.ring_scene(num_images=5, num_points=60, obs_per_point=3, seed=4)
    prob = tmp_path / "p.bin"
    write_problem(prob, s, 5)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin"), "--bad-size"],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stdout.startswith("err -1 status -2")


@pytest.mark.gpu
def test_facade_solve_matches_oracle(tmp_path):
    import oracle
    exe = build_facade(str(tmp_path))
    s = synthetic.config(0)
    prob = tmp_path / "p.bin"
    write_problem(prob, s, 20)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    x = np.fromfile(tmp_path / "x.bin", dtype=np.float64)
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(max_iterations=20, eps1=0.0,
                                                                    eps2=0.0))
    c = oracle.cost(s, x, s.near_y)
    assert abs(c - rref.final_cost) <= 1e-6 * rref.final_cost


def test_ceres_signature_refuses_fixed_cameras(tmp_path):
    # CameraSharedCeresOptimizor needs every group free (camera_shared_ceres_optimizor.hpp:193-202)
    exe = build_facade(str(tmp_path))
    s = synthetic.full_model_scene(seed=2, num_images=5, num_points=60, fix_mask=abi.FIX_CAMERAS,
                                   constraints=False, covariances=False)
    prob = tmp_path / "p.bin"
    write_problem(prob, s, 5, mode=2)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin")], capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stdout.startswith("err -1")


@pytest.mark.gpu
def test_ceres_signature_solve_matches_oracle(tmp_path):
    # the production caller's optimizer: free full-model cameras, Huber(1.0),
    # Ceres' stops, against the oracle run with the same options
    import oracle
    exe = build_facade(str(tmp_path))
    s = synthetic.full_model_scene(seed=4, num_images=12, num_points=500, num_cameras=1,
                                   fix_mask=0, constraints=False, covariances=False,
                                   obs_per_point=4)
    prob = tmp_path / "p.bin"
    write_problem(prob, s, 30, mode=1)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    x = np.fromfile(tmp_path / "x.bin", dtype=np.float64)
    assert x.shape == s.x0.shape
    opt = abi.make_options(max_iterations=30, eps1=1e-10, eps2=1e-8, loss=abi.LOSS_HUBER,
                           huber_delta=1.0, function_tolerance=1e-6)
    err, x_ref, rref = oracle.lm_solve(s, options=opt)
    assert err == 0
    toks = r.stdout.split()
    fields = dict(zip(toks[0::2], toks[1::2]))
    assert int(fields["iterations"]) == rref.iterations
    assert int(fields["stop"]) == rref.stop_reason
    c = oracle.cost(s, x, s.near_y, loss=abi.LOSS_HUBER, huber_delta=1.0)
    assert abs(c - rref.final_cost) <= 1e-9 * rref.final_cost


def test_gcp_facade_builds_and_rejects_bad_initial_x(tmp_path):
    exe = build_facade(str(tmp_path), "gcp_solve")
    s = synthetic.gcp_scene(seed=1, num_images=5, num_points=60, num_gcps=3)
    prob = tmp_path / "g.bin"
    write_gcp_problem(prob, s, 5)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin"), "--bad-size"],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stdout.startswith("err -1 status -2")


@pytest.mark.gpu
def test_gcp_facade_solve_matches_oracle(tmp_path):
    # BAGCPConstrainedLevenbergMarquardtOptimizor through the facade: the
    # naive layout in and out, control points last, against the oracle's
    # solve of the same problem with point priors
    import oracle
    exe = build_facade(str(tmp_path), "gcp_solve")
    s = synthetic.gcp_scene(seed=6, num_images=9, num_points=350, num_gcps=7)
    prob = tmp_path / "g.bin"
    perm = write_gcp_problem(prob, s, 30)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.fromfile(tmp_path / "x.bin", dtype=np.float64)
    C6, P3 = 6 * s.number_of_images, 3 * s.number_of_points
    xn, y0 = out[:C6 + P3], out[C6 + P3:]
    # back to the point-prior scene's layout [points][images]
    pts = np.empty((s.number_of_points, 3))
    pts[perm] = xn[C6:].reshape(-1, 3)
    x = np.concatenate([pts.reshape(-1), xn[:C6]])
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(max_iterations=30))
    assert err == 0 and rref.stop_reason == abi.STOP_SMALL_STEP
    c = oracle.cost(s, x, s.near_y)
    assert abs(c - rref.final_cost) <= 1e-9 * rref.final_cost
    # the facade's vector function at x0: keys, then the control points
    fmap = s.feature_maps
    y_ref = oracle.vector_function(s, s.x0)
    assert np.allclose(y0[:2 * s.number_of_keys], y_ref[:2 * s.number_of_keys], rtol=1e-13, atol=1e-15)
    np.testing.assert_array_equal(y0[2 * s.number_of_keys:], y_ref[2 * s.number_of_keys:])
    del fmap


def test_triangulation_facade_refuses_one_view(tmp_path):
    # MultipleViewMaximumLikelihoodEstimator needs two views (:66-69)
    exe = build_facade(str(tmp_path), "triangulate_solve")
    b = synthetic.triangulation_batch(seed=1, num_points=5)
    path = tmp_path / "t.bin"
    write_triangulation(path, b)
    r = subprocess.run([exe, str(path), str(tmp_path / "o.bin"), "--one-view"],
                       capture_output=True, text=True)
    assert r.returncode == 1 and r.stdout.startswith("mle -1")


@pytest.mark.gpu
def test_triangulation_facade_matches_oracle(tmp_path):
    import oracle
    exe = build_facade(str(tmp_path), "triangulate_solve")
    b = synthetic.triangulation_batch(seed=7, num_points=500, noise=0.5)
    path = tmp_path / "t.bin"
    write_triangulation(path, b)
    r = subprocess.run([exe, str(path), str(tmp_path / "o.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = (tmp_path / "o.bin").read_bytes()
    n = len(b.track_offsets) - 1
    pts = np.frombuffer(raw[:24 * n], dtype=np.float64).reshape(-1, 3)
    st = np.frombuffer(raw[24 * n:28 * n], dtype=np.int32)
    p0 = np.frombuffer(raw[28 * n:], dtype=np.float64)
    ref, sref = oracle.triangulate(b)
    assert np.array_equal(st, sref)
    # FP64 on both sides; the device contracts multiply-adds (see
    # tests/test_gpu_triangulate.py): points within 1e-6
    assert np.max(np.abs(pts - ref)) < 1e-6
    assert np.array_equal(p0, pts[0])


@pytest.mark.gpu
def test_facade_images_only_solve_matches_oracle(tmp_path):
    """The facade with points and cameras fixed (set_fix_points,
    set_fix_cameras): x holds the images only, as the reference's
    (camera_shared_vector_function.hpp:349-410), and the solve reaches the
    oracle's final cost (SolveImagesCamerasOnly,
    camera_shared_normal_equation_solver.hpp:540-706)."""
    import oracle
    exe = build_facade(str(tmp_path))
    s = synthetic.ring_scene(num_images=8, num_points=300, obs_per_point=4, seed=14,
                             fix_mask=abi.FIX_POINTS | abi.FIX_CAMERAS)
    assert len(s.x0) == 6 * s.number_of_images
    prob = tmp_path / "p.bin"
    write_problem(prob, s, 10, mode=3)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    x = np.fromfile(tmp_path / "x.bin", dtype=np.float64)
    assert len(x) == 6 * s.number_of_images
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(max_iterations=10, eps1=0.0,
                                                                    eps2=0.0))
    assert err == 0
    assert abs(oracle.cost(s, x, s.near_y) - rref.final_cost) <= 1e-9 * rref.final_cost


def test_facade_images_only_rejects_bad_initial_x(tmp_path):
    """With points and cameras fixed the facade expects x0 of 6 I values and
    refuses one short of it, before any device work."""
    exe = build_facade(str(tmp_path))
    s = synthetic.ring_scene(num_images=5, num_points=60, obs_per_point=3, seed=4,
                             fix_mask=abi.FIX_POINTS | abi.FIX_CAMERAS)
    prob = tmp_path / "p.bin"
    write_problem(prob, s, 5, mode=3)
    r = subprocess.run([exe, str(prob), str(tmp_path / "x.bin"), "--bad-size"],
                       capture_output=True, text=True)
    assert r.returncode == 1
    assert r.stdout.startswith("err -1 status -2")
