"""Soft constraints on points and images on the device path against the
oracle: the constraint rows of y, the cost, the Schur step and full solves
(rows = parameter copies with per-row weights, camera_shared_vector_function.hpp:483-629;
normal-equation terms, camera_shared_normal_equation_builder.hpp:309-349,418-459)."""
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


def constrained(seed=3, num_images=10, num_points=400):
    s = synthetic.full_model_scene(seed=seed, num_images=num_images, num_points=num_points,
                                   fix_mask=abi.FIX_CAMERAS, constraints=True, obs_per_point=4)
    assert s.point_constraints and s.image_constraints
    return s


def test_vector_function_constraint_rows(gba):
    s = constrained()
    y = gba.vector_function(s, s.x0)
    y_ref = oracle.vector_function(s, s.x0)
    assert y.shape == y_ref.shape and len(y) > 2 * s.number_of_keys
    np.testing.assert_allclose(y, y_ref, rtol=1e-13, atol=1e-9)


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_cost_with_constraints(gba, precision):
    s = constrained()
    c = gba.cost(s, s.x0, options=abi.make_options(precision=precision))
    c_ref = oracle.cost(s, s.x0, s.near_y)
    assert abs(c - c_ref) <= 1e-11 * c_ref, (c, c_ref)


def test_schur_step_with_constraints(gba):
    s = constrained()
    N, g = oracle.normal_equation_dense(s, s.x0, s.near_y)
    mu = 1e-3 * float(np.max(np.diag(N)))
    dx = gba.schur_step(s, s.x0, mu, options=abi.make_options())
    err, dref = oracle.schur_step(s, s.x0, s.near_y, mu, faithful=False)
    assert err == 0
    assert np.linalg.norm(dx - dref) / np.linalg.norm(dref) < 1e-9


@pytest.mark.parametrize("precision", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
@pytest.mark.parametrize("solver", [abi.LINEAR_DENSE_CHOLESKY, abi.LINEAR_PCG])
def test_lm_with_constraints_matches_oracle(gba, precision, solver):
    s = constrained(seed=5)
    opt = abi.make_options(max_iterations=15, eps1=0.0, eps2=0.0, precision=precision,
                           linear_solver=solver, pcg_relative_tolerance=1e-10,
                           pcg_max_iterations=300)
    x, rep = gba.solve(s, opt)
    err, x_ref, rref = oracle.lm_solve(s, options=abi.make_options(
        max_iterations=15, eps1=0.0, eps2=0.0))
    assert err == 0 and rep.status == abi.GBA_OK
    assert abs(rep.final_cost - rref.final_cost) <= 1e-6 * rref.final_cost, \
        (rep.final_cost, rref.final_cost)
    assert abs(rep.final_rmse - rref.final_rmse) <= 1e-4


def test_constraint_bad_index(gba):
    s = constrained()
    s.point_constraints = list(s.point_constraints) + [(s.number_of_points + 3, 1)]
    s.near_y = np.concatenate([s.near_y, [0.0]])
    if s.constraint_weights is not None:
        s.constraint_weights = np.concatenate([s.constraint_weights, [1.0]])
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s, abi.make_options(max_iterations=2))
    assert e.value.status == abi.GBA_ERR_BAD_INDEX
