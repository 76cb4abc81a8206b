"""Point priors (the ground control points of the GCP-constrained model) on
the device path against the oracle: prior rows of y, the cost, the Schur
step and full LM solves (ba_gcp_constrained_vector_function.hpp:60-110,
ba_gcp_constrained_normal_equation_builder.hpp:42-75,
ba_gcp_constrained_mahalanobis_distance_calculator.hpp:28-62)."""
import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def test_vector_function_prior_rows(gba):
    s = synthetic.gcp_scene(seed=1, num_images=8, num_points=300, num_gcps=6)
    y = gba.vector_function(s, s.x0)
    y_ref = oracle.vector_function(s, s.x0)
    assert y.shape == y_ref.shape
    np.testing.assert_allclose(y, y_ref, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_cost_with_priors(gba, precision):
    s = synthetic.gcp_scene(seed=1, num_images=8, num_points=300, num_gcps=6)
    c = gba.cost(s, s.x0, options=abi.make_options(precision=precision))
    c_ref = oracle.cost(s, s.x0, s.near_y)
    assert abs(c - c_ref) <= 1e-11 * c_ref, (c, c_ref)


def test_schur_step_with_priors(gba):
    s = synthetic.gcp_scene(seed=3, num_images=8, num_points=300, num_gcps=6)
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    mu = 1e-3 * float(np.max(np.diag(N)))
    dx = gba.schur_step(s, s.x0, mu, options=abi.make_options())
    err, dref = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=False)
    assert err == 0
    assert np.linalg.norm(dx - dref) / np.linalg.norm(dref) < 1e-9


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
@pytest.mark.parametrize("solver", [abi.LINEAR_DENSE_CHOLESKY, abi.LINEAR_PCG])
def test_lm_with_priors_matches_oracle(gba, precision, solver):
    s = synthetic.gcp_scene(seed=2, num_images=10, num_points=400, num_gcps=8)
    opt = dict(max_iterations=30)
    x, rep = gba.solve(s, abi.make_options(precision=precision, linear_solver=solver,
                                           pcg_relative_tolerance=1e-10,
                                           pcg_max_iterations=300, **opt))
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(**opt))
    assert err == 0 and rep.status == abi.GBA_OK
    # converged solves (small step): the same minimum
    assert rref.stop_reason == abi.STOP_SMALL_STEP
    assert abs(rep.final_cost - rref.final_cost) <= 1e-6 * rref.final_cost, \
        (rep.final_cost, rref.final_cost)
    np.testing.assert_allclose(x[:3 * s.number_of_points], x_ref[:3 * s.number_of_points],
                               rtol=0, atol=1e-5)


def test_batch_with_priors_equals_alone(gba):
    scenes = [synthetic.gcp_scene(seed=10 + i, num_images=6 + i, num_points=200 + 50 * i,
                                  num_gcps=4 + i) for i in range(3)]
    scenes.append(synthetic.config(0))   # a problem without priors in the same batch
    opt = abi.make_options(max_iterations=10, eps1=0.0, eps2=0.0)
    xs, reps = gba.solve_batch(scenes, opt)
    for s, x, r in zip(scenes, xs, reps):
        x1, r1 = gba.solve(s, opt)
        assert np.array_equal(x, x1) and r.final_cost == r1.final_cost


def test_prior_bad_index(gba):
    s = synthetic.gcp_scene(seed=1, num_images=6, num_points=80, num_gcps=3)
    s.point_priors = [0, 1, s.number_of_points + 2]
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s, abi.make_options(max_iterations=2))
    assert e.value.status == abi.GBA_ERR_BAD_INDEX
