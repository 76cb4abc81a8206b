"""The two schedules of the dense factorization give the same bits: the
single-launch dataflow factorization (one problem alone on the device) and
the per-column launches (batches, or shared_device=1), on systems of one to
many tile columns, in both precisions."""
import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
@pytest.mark.parametrize("images", [3, 6, 11, 40, 75])
def test_dataflow_equals_per_column_schedule(precision, images):
    from hs_sfm_gb300 import gba
    s = synthetic.ring_scene(num_images=images, num_points=60 * images, obs_per_point=4,
                             seed=100 + images)
    opt = dict(max_iterations=6, precision=precision, eps1=0.0, eps2=0.0)
    x_df, r_df = gba.solve(s, abi.make_options(**opt))
    x_pc, r_pc = gba.solve(s, abi.make_options(shared_device=1, **opt))
    assert r_df.status == abi.GBA_OK and r_pc.status == abi.GBA_OK
    assert r_df.accepted == r_pc.accepted
    assert np.array_equal(x_df, x_pc)
    other = synthetic.ring_scene(num_images=5, num_points=200, seed=7)
    xs, reps = gba.solve_batch([s, other], abi.make_options(**opt))
    assert np.array_equal(xs[0], x_df)


@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_dataflow_repeated_runs_and_graph(precision):
    """Epochs advance launch after launch: a resident plan re-run (graph
    replay) gives the same x each time."""
    from hs_sfm_gb300 import gba
    s = synthetic.ring_scene(num_images=50, num_points=3000, seed=5)
    p = gba.Plan(s, abi.make_options(max_iterations=5, precision=precision, eps1=0.0, eps2=0.0))
    xs = []
    for _ in range(3):
        p.run()
        p.synchronize()
        xs.append(p.x(0))
        assert p.report(0).status == abi.GBA_OK
    p.close()
    assert np.array_equal(xs[0], xs[1]) and np.array_equal(xs[1], xs[2])



@pytest.mark.parametrize("images", [3, 6, 11, 25, 42])
def test_small_system_kernel_equals_per_column_launches(images, monkeypatch):
    """Batches of small systems (at most eight tile rows, mixed precision)
    factor and solve in one launch per iteration (k_chol_small) with the
    per-element arithmetic of the per-column launches: the same bits as
    those (GBA_CHOL_COLUMNS=1) and as the dataflow factorization alone."""
    from hs_sfm_gb300 import gba
    s = synthetic.ring_scene(num_images=images, num_points=60 * images, obs_per_point=4,
                             seed=200 + images)
    other = synthetic.ring_scene(num_images=7, num_points=300, seed=9)
    opt = abi.make_options(max_iterations=6, precision=abi.PRECISION_MIXED, eps1=0.0, eps2=0.0)
    x_df, r_df = gba.solve(s, opt)
    xs, reps = gba.solve_batch([s, other], opt)
    monkeypatch.setenv("GBA_CHOL_COLUMNS", "1")
    xc, repc = gba.solve_batch([s, other], opt)
    monkeypatch.delenv("GBA_CHOL_COLUMNS")
    for a, b in zip(xs, xc):
        assert np.array_equal(a, b)
    assert np.array_equal(xs[0], x_df)
    assert reps[0].final_cost == repc[0].final_cost == r_df.final_cost
