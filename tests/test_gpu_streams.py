"""An LM iteration forks: the image sums and the after-linearization control
of the previous linearization run on a second stream beside the point Schur
and the key-pair assembly.  The fork changes no arithmetic, so every solve
gives the same bits, reports and stop reasons as the one-stream order
(GBA_ONE_STREAM=1), also when problems stop early (small gradient or step)
while the next iteration's point Schur already ran for them, and when a
factorization fails."""
import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def _both(gba, monkeypatch, scenes, opt):
    xs, reps = gba.solve_batch(scenes, opt)
    monkeypatch.setenv("GBA_ONE_STREAM", "1")
    xo, repo = gba.solve_batch(scenes, opt)
    monkeypatch.delenv("GBA_ONE_STREAM")
    for a, b, ra, rb in zip(xs, xo, reps, repo):
        np.testing.assert_array_equal(a, b)
        assert ra.final_cost == rb.final_cost
        assert (ra.iterations, ra.accepted, ra.rejected, ra.stop_reason, ra.status) == \
               (rb.iterations, rb.accepted, rb.rejected, rb.stop_reason, rb.status)
    return reps


@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_fork_same_bits_dense(gba, monkeypatch, precision):
    scenes = [synthetic.ring_scene(num_images=10, num_points=800, obs_range=(3, 8), seed=s) for s in (1, 2)]
    scenes.append(synthetic.grid_scene(num_images=30, num_points=3000, seed=4))
    _both(gba, monkeypatch, scenes, abi.make_options(max_iterations=8, eps1=0.0, eps2=0.0,
                                                     precision=precision))


def test_fork_same_bits_early_stops(gba, monkeypatch):
    """Stopping tests on: the problems stop at different iterations."""
    scenes = [synthetic.ring_scene(num_images=8, num_points=500, seed=s) for s in (3, 4, 5)]
    reps = _both(gba, monkeypatch, scenes, abi.make_options(max_iterations=40, eps1=1e-6, eps2=1e-10,
                                                            precision=abi.PRECISION_FP64))
    assert any(r.iterations < 40 for r in reps)


def test_fork_same_bits_pcg(gba, monkeypatch):
    scenes = [synthetic.walk_scene(num_images=50, num_points=3000, mean_obs=8.0, seed=s,
                                   outlier_fraction=0.01, max_track=30) for s in (6, 7)]
    _both(gba, monkeypatch, scenes, abi.make_options(max_iterations=5, eps1=0.0, eps2=0.0,
                                                     precision=abi.PRECISION_MIXED,
                                                     linear_solver=abi.LINEAR_PCG,
                                                     loss=abi.LOSS_HUBER, huber_delta=1.0))


def test_fork_same_bits_free_cameras(gba, monkeypatch):
    s = synthetic.full_model_scene(seed=3, num_images=8, num_points=300, num_cameras=2, fix_mask=0)
    _both(gba, monkeypatch, [s], abi.make_options(max_iterations=6, eps1=0.0, eps2=0.0,
                                                  precision=abi.PRECISION_FP64))
