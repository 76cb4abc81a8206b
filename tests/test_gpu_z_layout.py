"""The Schur assembly's per-key records (Z = C_p^-1 J_p^T J_i) in either
layout: records in key order or image-major planes of value pairs.  Only
where the records lie changes, so every solve gives the same bits in both,
on the dense and the PCG solver, with free cameras (camera records in the
planes too), and a batch whose plan picks one layout matches each problem
solved alone with the other."""
import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def _same(gba, scene, **kw):
    outs = []
    for layout in (abi.Z_RECORDS, abi.Z_PLANES):
        x, rep = gba.solve(scene, abi.make_options(z_layout=layout, eps1=0.0, eps2=0.0, **kw))
        assert rep.status == abi.GBA_OK
        outs.append((x, rep))
    (xa, ra), (xb, rb) = outs
    np.testing.assert_array_equal(xa, xb)
    assert ra.final_cost == rb.final_cost
    assert ra.accepted == rb.accepted
    return ra


@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_dense_solver_same_bits(gba, precision):
    s = synthetic.ring_scene(num_images=24, num_points=3000, obs_range=(3, 8), seed=41)
    rep = _same(gba, s, max_iterations=8, precision=precision)
    assert rep.final_cost < rep.initial_cost


def test_grid_same_bits(gba):
    s = synthetic.grid_scene(num_images=40, num_points=5000, seed=8)
    _same(gba, s, max_iterations=6, precision=abi.PRECISION_MIXED)


def test_pcg_same_bits(gba):
    s = synthetic.walk_scene(num_images=60, num_points=4000, mean_obs=8.0, seed=7,
                             outlier_fraction=0.01, max_track=30)
    _same(gba, s, max_iterations=5, precision=abi.PRECISION_MIXED, linear_solver=abi.LINEAR_PCG,
          loss=abi.LOSS_HUBER, huber_delta=1.0)


@pytest.mark.parametrize("linear_solver", [abi.LINEAR_DENSE_CHOLESKY, abi.LINEAR_PCG])
def test_free_cameras_same_bits(gba, linear_solver):
    s = synthetic.full_model_scene(seed=3, num_images=8, num_points=300, num_cameras=2, fix_mask=0)
    _same(gba, s, max_iterations=6, precision=abi.PRECISION_FP64, linear_solver=linear_solver)


def test_batch_in_one_layout_equals_alone_in_the_other(gba):
    scenes = [synthetic.ring_scene(num_images=12, num_points=1500, obs_range=(3, 8), seed=s) for s in (5, 6)]
    scenes.append(synthetic.grid_scene(num_images=30, num_points=3000, seed=9))
    opt = dict(max_iterations=6, eps1=0.0, eps2=0.0, precision=abi.PRECISION_MIXED)
    xs, reps = gba.solve_batch(scenes, abi.make_options(z_layout=abi.Z_PLANES, **opt))
    for sc, xb, rb in zip(scenes, xs, reps):
        xa, ra = gba.solve(sc, abi.make_options(z_layout=abi.Z_RECORDS, **opt))
        np.testing.assert_array_equal(xa, xb)
        assert ra.final_cost == rb.final_cost


def test_invalid_layout_is_refused(gba):
    s = synthetic.ring_scene(num_images=6, num_points=200, seed=1)
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s, abi.make_options(z_layout=3))
    assert e.value.status == abi.GBA_ERR_INVALID


def test_structure_reports_the_layout_and_the_fork(gba):
    """gba_plan_structure says which layout and schedule a plan took: planes
    for dense windows, records for the sparse grid; the iteration forks
    only in plans of at least 300k keys; small batches factor in the
    small-system kernel, one problem in the dataflow launch."""
    wins = [synthetic.ring_scene(num_images=12, num_points=1500, obs_range=(3, 8), seed=s) for s in (5, 6)]
    grid = synthetic.grid_scene(num_images=200, num_points=100000, seed=1)   # the bench's grid
    opt = abi.make_options(max_iterations=2, precision=abi.PRECISION_MIXED)
    p = gba.Plan(wins, opt)
    st = p.structure()
    p.close()
    assert st["z_layout"] == abi.Z_PLANES and st["forked"] == 0 and st["factor_schedule"] == 2
    assert grid.number_of_keys >= 300_000
    p = gba.Plan(grid, opt)
    st = p.structure()
    p.close()
    assert st["z_layout"] == abi.Z_RECORDS and st["forked"] == 1 and st["factor_schedule"] == 1
    p = gba.Plan(grid, abi.make_options(max_iterations=2, precision=abi.PRECISION_MIXED, z_layout=abi.Z_PLANES))
    assert p.structure()["z_layout"] == abi.Z_PLANES
    p.close()
