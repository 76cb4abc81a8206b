"""Every fix mask of the reference on the device: points, images and shared
cameras fixed in all combinations but all three.  The reference serves them
through ComputeReducedSystem / SolvePointsOnly / SolveImagesCamerasOnly
(camera_shared_normal_equation_solver.hpp:75-114,540-706) and its own solver
test runs each mask (unit_test/bundle_adjustment/
test_camera_shared_normal_equation_solver.cpp:185-211).  On the device a
fixed group keeps its values with zero Jacobian columns, which leaves the
same damped system for the free unknowns.  Checked against the CPU FP64
oracle on the full model (several cameras, every intrinsic group, soft
constraints, per-key covariances): the Schur step and the LM solve to 1e-9
relative on the FP64 path, the mixed path by the acceptance rule."""
import numpy as np
import pytest

import oracle
from helpers import ALL_FIX_MASKS, full_scene
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-9


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def scene(fix_mask, seed=7):
    return full_scene(fix_mask, seed=seed, num_images=8, num_points=200, obs_per_point=4)


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
def test_schur_step_every_fix_mask(gba, fix_mask):
    s = scene(fix_mask)
    assert len(s.x0) == abi.x_size(s)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    mu = 1e-3 * float(np.max(np.diag(N)))
    dx = gba.schur_step(s, s.x0, mu)
    err, dref = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=False)
    assert err == 0
    assert np.linalg.norm(dx - dref) <= FP64_RTOL * np.linalg.norm(dref), fix_mask
    # the reference's own property: (N + mu I) delta = g
    r = (N + mu * np.eye(len(g))) @ dx - g
    assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(g)


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
def test_lm_every_fix_mask_fp64(gba, fix_mask):
    s = scene(fix_mask)
    opt = abi.make_options(max_iterations=10, eps1=0.0, eps2=0.0)
    x, rep = gba.solve(s, opt)
    err, x_ref, rref = oracle.lm_solve(s, options=opt)
    assert err == 0 and rep.status == abi.GBA_OK
    assert rep.final_cost < rep.initial_cost
    assert abs(rep.final_cost - rref.final_cost) <= FP64_RTOL * rref.final_cost, \
        (fix_mask, rep.final_cost, rref.final_cost)
    # (accept / reject counts may differ once converged: a step whose cost
    # change is at the rounding floor goes either way)
    np.testing.assert_allclose(x, x_ref, rtol=1e-7, atol=1e-8)


@pytest.mark.parametrize("fix_mask", ALL_FIX_MASKS)
def test_lm_every_fix_mask_mixed(gba, fix_mask):
    # twice the views of the FP64 test: the full model on the tiny scene has
    # a flat valley of the free intrinsics in which FP32 and FP64
    # trajectories part (test_gpu_free_cameras.py)
    s = full_scene(fix_mask, seed=9, num_images=16, num_points=600, obs_per_point=5)
    opt = abi.make_options(max_iterations=10, eps1=0.0, eps2=0.0, precision=abi.PRECISION_MIXED)
    x, rep = gba.solve(s, opt)
    err, _, rref = oracle.lm_solve(s, options=abi.make_options(max_iterations=10, eps1=0.0, eps2=0.0))
    assert err == 0 and rep.status == abi.GBA_OK
    assert abs(rep.final_cost - rref.final_cost) <= 1e-6 * rref.final_cost, \
        (fix_mask, rep.final_cost, rref.final_cost)
    assert abs(rep.final_rmse - rref.final_rmse) <= 1e-4


@pytest.mark.parametrize("fix_mask", [abi.FIX_CAMERAS, abi.FIX_POINTS | abi.FIX_CAMERAS,
                                      abi.FIX_IMAGES | abi.FIX_CAMERAS])
def test_pcg_fixed_groups(gba, fix_mask):
    """The block-Jacobi PCG solver with fixed points or images (cameras
    fixed): the same LM result as the oracle's exact solve."""
    s = synthetic.ring_scene(num_images=12, num_points=600, obs_per_point=4, seed=13,
                             fix_mask=fix_mask)
    opt = dict(max_iterations=8, eps1=0.0, eps2=0.0)
    x, rep = gba.solve(s, abi.make_options(linear_solver=abi.LINEAR_PCG, pcg_max_iterations=200,
                                           pcg_relative_tolerance=1e-12, **opt))
    err, _, rref = oracle.lm_solve(s, options=abi.make_options(**opt))
    assert err == 0 and rep.status == abi.GBA_OK
    assert abs(rep.final_cost - rref.final_cost) <= 1e-8 * rref.final_cost


def test_fixed_groups_keep_their_values_in_a_batch(gba):
    """A batch mixing fix masks: each problem's x has the caller's layout
    (fixed groups dropped), and its result is the same alone and in the mix."""
    scenes = [scene(m, seed=20 + m) for m in ALL_FIX_MASKS]
    opt = abi.make_options(max_iterations=6, eps1=0.0, eps2=0.0)
    xs, reps = gba.solve_batch(scenes, opt)
    for s, x, r in zip(scenes, xs, reps):
        assert len(x) == abi.x_size(s)
        xa, ra = gba.solve(s, opt)
        assert r.status == abi.GBA_OK and ra.final_cost == r.final_cost
        np.testing.assert_array_equal(x, xa)


def test_all_groups_fixed_is_refused(gba):
    s = scene(abi.FIX_POINTS | abi.FIX_IMAGES | abi.FIX_CAMERAS)
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s, abi.make_options(max_iterations=2))
    assert e.value.status == abi.GBA_ERR_UNSUPPORTED
