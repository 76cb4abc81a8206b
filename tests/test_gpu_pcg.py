"""Block-Jacobi PCG on the block-sparse reduced system against the oracle's
exact Schur solve: the step itself (FP64 at a tight tolerance), LM solves on
random-walk scenes with outliers under Huber (the large-scene workload in
small), batch-vs-alone equality, and scenes above the dense limit."""
import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6
RMSE_ATOL = 1e-4


def pcg_opts(precision=abi.PRECISION_FP64, iters=10, tol=1e-6, pcg_iters=200, **kw):
    return abi.make_options(max_iterations=iters, eps1=0.0, eps2=0.0, precision=precision,
                            linear_solver=abi.LINEAR_PCG, pcg_max_iterations=pcg_iters,
                            pcg_relative_tolerance=tol, **kw)


def small_walk(num_images=120, num_points=8000, seed=31, outliers=0.01):
    return synthetic.walk_scene(num_images=num_images, num_points=num_points, mean_obs=8.0,
                                seed=seed, outlier_fraction=outliers, max_track=30)


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def test_pcg_step_matches_exact_schur_step(gba):
    s = synthetic.ring_scene(num_images=30, num_points=900, obs_per_point=5, seed=12)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    for mu in (float(np.max(np.diag(N))), 1e-2 * float(np.max(np.diag(N)))):
        dx = gba.schur_step(s, s.x0, mu, options=pcg_opts(tol=1e-13, pcg_iters=400))
        err, dref = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=False)
        assert err == 0
        rel = np.linalg.norm(dx - dref) / np.linalg.norm(dref)
        assert rel < 1e-8, rel


def test_pcg_lm_matches_oracle_fp64(gba):
    """Converged inner solves: the LM trajectory is the oracle's."""
    s = synthetic.ring_scene(num_images=30, num_points=900, obs_per_point=5, seed=12)
    x, rep = gba.solve(s, pcg_opts(iters=15, tol=1e-9, pcg_iters=300))
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(max_iterations=15, eps1=0.0, eps2=0.0))
    assert err == 0 and rep.status == abi.GBA_OK
    assert abs(rep.final_cost - rref.final_cost) <= 1e-8 * rref.final_cost
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_pcg_huber_outliers_matches_oracle(gba, precision):
    """The large-scene configuration in small: outliers under Huber, inner
    relative tolerance 1e-6, final cost within the acceptance tolerance."""
    s = synthetic.ring_scene(num_images=16, num_points=1500, obs_per_point=5, seed=21)
    rng = np.random.default_rng(21)
    y = s.near_y.reshape(-1, 2).copy()
    out = rng.random(len(y)) < 0.01
    y[out] = np.stack([rng.uniform(0, 1920, out.sum()), rng.uniform(0, 1080, out.sum())], 1)
    s.near_y = y.reshape(-1)
    x, rep = gba.solve(s, pcg_opts(precision, iters=20, tol=1e-6, pcg_iters=200,
                                   loss=abi.LOSS_HUBER, huber_delta=1.0))
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(
        max_iterations=20, eps1=0.0, eps2=0.0, loss=abi.LOSS_HUBER, huber_delta=1.0))
    assert err == 0 and rep.status == abi.GBA_OK and rep.pcg_iterations > 0
    assert abs(rep.final_cost - rref.final_cost) <= COST_RTOL * rref.final_cost, \
        (rep.final_cost, rref.final_cost)
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_pcg_walk_descends(gba, precision):
    """A random walk with 1% outliers: every accepted step lowers the cost and
    the solve ends within 1% of the exact-step solve after the same number
    of iterations (inner solves stop at 1e-6 or 200 iterations)."""
    s = small_walk()
    H = dict(loss=abi.LOSS_HUBER, huber_delta=1.0)
    x, rep = gba.solve(s, pcg_opts(precision, iters=12, **H))
    xd, rd = gba.solve(s, abi.make_options(max_iterations=12, eps1=0.0, eps2=0.0, **H))
    assert rep.status == abi.GBA_OK and rep.accepted > 0
    assert rep.final_cost < 0.7 * rep.initial_cost
    assert rep.final_cost <= 1.01 * rd.final_cost, (rep.final_cost, rd.final_cost)


def test_pcg_breakdown_keeps_the_step(gba):
    """A tolerance below the rounding floor ends the inner solve at the
    breakdown instead of wandering: the step is still the exact one."""
    s = synthetic.ring_scene(num_images=30, num_points=900, obs_per_point=5, seed=12)
    xd, rd = gba.solve(s, abi.make_options(max_iterations=1, eps1=0.0, eps2=0.0))
    x, rep = gba.solve(s, pcg_opts(iters=1, tol=1e-14, pcg_iters=1000))
    assert rep.accepted == 1
    assert abs(rep.final_cost - rd.final_cost) <= 1e-9 * rd.final_cost
    assert rep.pcg_iterations < 1000


def test_pcg_dense_agree_on_grid(gba):
    s = synthetic.grid_scene(num_images=40, num_points=5000, seed=8)
    xd, rd = gba.solve(s, abi.make_options(max_iterations=10, eps1=0.0, eps2=0.0))
    xp, rp = gba.solve(s, pcg_opts(iters=10, tol=1e-12, pcg_iters=400))
    assert abs(rp.final_cost - rd.final_cost) <= 1e-9 * rd.final_cost


def test_pcg_batch_equals_alone_bitwise(gba):
    scenes = [small_walk(num_images=40, num_points=2000, seed=s) for s in (1, 2, 3)]
    opt = pcg_opts(abi.PRECISION_MIXED, iters=6)
    xs, reps = gba.solve_batch(scenes, opt)
    for sc, xb, rb in zip(scenes, xs, reps):
        xa, ra = gba.solve(sc, opt)
        assert ra.final_cost == rb.final_cost
        assert ra.pcg_iterations == rb.pcg_iterations
        np.testing.assert_array_equal(xa, xb)


def test_pcg_beyond_the_dense_limit(gba):
    s = small_walk(num_images=2100, num_points=12000, seed=5, outliers=0.0)
    dense = abi.make_options(max_iterations=2)
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s, dense)
    assert e.value.status == abi.GBA_ERR_UNSUPPORTED
    x, rep = gba.solve(s, pcg_opts(abi.PRECISION_MIXED, iters=4))
    assert rep.status == abi.GBA_OK
    assert rep.final_cost < rep.initial_cost


@pytest.mark.parametrize("pcg_iters,tol", [(200, 1e-6), (7, 1e-14)])
def test_pcg_device_loop_equals_unrolled_launches(gba, monkeypatch, pcg_iters, tol):
    """In a CUDA graph the PCG iterations run as a while node (two iterations
    and a control kernel per pass, ending once every problem's inner solve
    has stopped): the same bits as one launch pair per iteration
    (GBA_PCG_UNROLLED=1), with fewer launches once the solves converge.  An
    odd iteration cap ends the loop mid-pass."""
    scenes = [small_walk(num_images=40, num_points=2000, seed=s) for s in (4, 5)]
    opt = pcg_opts(abi.PRECISION_MIXED, iters=5, tol=tol, pcg_iters=pcg_iters)
    k0 = gba.kernel_launch_count()
    xs, reps = gba.solve_batch(scenes, opt)
    k_loop = gba.kernel_launch_count() - k0
    monkeypatch.setenv("GBA_PCG_UNROLLED", "1")
    k0 = gba.kernel_launch_count()
    xu, repu = gba.solve_batch(scenes, opt)
    k_unrolled = gba.kernel_launch_count() - k0
    monkeypatch.delenv("GBA_PCG_UNROLLED")
    for a, b, ra, rb in zip(xs, xu, reps, repu):
        np.testing.assert_array_equal(a, b)
        assert ra.final_cost == rb.final_cost
        assert ra.pcg_iterations == rb.pcg_iterations
    if tol > 1e-10:
        assert k_loop < k_unrolled
