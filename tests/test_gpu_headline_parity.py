"""Parity at the benchmarked sizes: the exact scenes bench.py times, solved on
the GPU and by the CPU FP64 oracle (point-major mode, the reference's
Schur-complement algorithm with its loops reordered by point), compared by
the acceptance rule of every result -- final cost within 1e-6 relative and
reprojection RMSE within 1e-4 px of the oracle.

* the grid of 200 cameras / 100,000 points / ~800k keys (radial distortion
  and intrinsics fixed), 20 LM iterations with the stopping tests off, on the
  mixed FP32/FP64 path and the plain FP64 path;
* windows of the 512-window batch (I ~ U{5..40}, P ~ U{500..20000}), solved
  together in one batched plan, 10 LM iterations each.  bench.py checks all
  512 of them outside its timed region; this test checks every 16th.

The oracle follows camera_shared_normal_equation_solver.hpp:75-538 (reduced
system, dense solve, back-substitution) and the LM schedule of Madsen,
Nielsen & Tingleff (2004) Alg. 3.16."""
from concurrent.futures import ThreadPoolExecutor
import os

import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-6
RMSE_ATOL = 1e-4
GRID_ITERS = 20
WINDOW_ITERS = 10


def _opts(precision, iters):
    return abi.make_options(max_iterations=iters, eps1=0.0, eps2=0.0, precision=precision)


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


@pytest.fixture(scope="module")
def grid():
    # bench.py's default workload (make_scene: seed 1, name cfg1)
    s = synthetic.grid_scene(num_images=200, num_points=100_000, seed=1, name="cfg1")
    err, x_ref, rref = oracle.lm_solve(s, options=_opts(abi.PRECISION_FP64, GRID_ITERS))
    assert err == 0
    return s, x_ref, rref


@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64],
                         ids=["mixed", "fp64"])
def test_headline_grid_matches_oracle(gba, grid, precision):
    s, x_ref, rref = grid
    assert s.number_of_keys > 790_000
    x, rep = gba.solve(s, _opts(precision, GRID_ITERS))
    assert rep.status == 0 and rep.iterations == GRID_ITERS
    rel = abs(rep.final_cost - rref.final_cost) / rref.final_cost
    assert rel <= COST_RTOL, (rep.final_cost, rref.final_cost, rel)
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL, (rep.final_rmse, rref.final_rmse)
    if precision == abi.PRECISION_FP64:
        assert rep.accepted == rref.accepted


def test_headline_free_intrinsics_grid_matches_oracle(gba):
    """The same grid with the shared camera free (radial + intrinsic
    parameters, 1,212 reduced-system unknowns), as bench.py times it: the
    mixed path by the acceptance rule."""
    s = synthetic.config(1, fix_mask=0)
    err, _, rref = oracle.lm_solve(s, options=_opts(abi.PRECISION_FP64, GRID_ITERS))
    assert err == 0
    x, rep = gba.solve(s, _opts(abi.PRECISION_MIXED, GRID_ITERS))
    assert rep.status == 0
    rel = abs(rep.final_cost - rref.final_cost) / rref.final_cost
    assert rel <= COST_RTOL, (rep.final_cost, rref.final_cost, rel)
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL


def test_headline_windows_match_oracle(gba):
    wins = synthetic.window_batch(num_windows=512, seed=3)[::16]
    xs, reps = gba.solve_batch(wins, _opts(abi.PRECISION_MIXED, WINDOW_ITERS))
    opt = _opts(abi.PRECISION_FP64, WINDOW_ITERS)
    with ThreadPoolExecutor(max(1, min(16, os.cpu_count() or 1))) as ex:
        refs = list(ex.map(lambda w: oracle.lm_solve(w, options=opt), wins))
    worst = 0.0
    for w, r, (err, _, rr) in zip(wins, reps, refs):
        assert err == 0 and r.status == 0, w.name
        rel = abs(r.final_cost - rr.final_cost) / rr.final_cost
        worst = max(worst, rel)
        assert rel <= COST_RTOL, (w.name, r.final_cost, rr.final_cost)
        assert abs(r.final_rmse - rr.final_rmse) <= RMSE_ATOL, w.name
    assert np.isfinite(worst)


def test_walk_at_a_tenth_pcg_huber_matches_oracle(gba):
    """The random-walk workload (block-Jacobi PCG, Huber 1 px, 1% outliers)
    at a tenth of the benchmarked size -- 200 cameras, 100,000 points -- so
    the oracle's dense solve of its 1,200 unknowns fits a test: the mixed
    path with the bench's PCG settings (relative residual 1e-6, at most 100
    iterations) by the acceptance rule, and an FP64 PCG solved to 1e-12
    against the oracle's exact steps to 1e-8."""
    s = synthetic.walk_scene(num_images=200, num_points=100_000, seed=2)
    common = dict(max_iterations=WINDOW_ITERS, eps1=0.0, eps2=0.0, loss=abi.LOSS_HUBER, huber_delta=1.0)
    err, _, rref = oracle.lm_solve(s, options=abi.make_options(**common))
    assert err == 0
    _, rep = gba.solve(s, abi.make_options(precision=abi.PRECISION_MIXED, linear_solver=abi.LINEAR_PCG,
                                           pcg_relative_tolerance=1e-6, pcg_max_iterations=100, **common))
    rel = abs(rep.final_cost - rref.final_cost) / rref.final_cost
    assert rep.status == 0 and rel <= COST_RTOL, (rep.final_cost, rref.final_cost, rel)
    assert abs(rep.final_rmse - rref.final_rmse) <= RMSE_ATOL
    _, r64 = gba.solve(s, abi.make_options(precision=abi.PRECISION_FP64, linear_solver=abi.LINEAR_PCG,
                                           pcg_relative_tolerance=1e-12, pcg_max_iterations=1000, **common))
    assert abs(r64.final_cost - rref.final_cost) <= 1e-8 * rref.final_cost, (r64.final_cost, rref.final_cost)
