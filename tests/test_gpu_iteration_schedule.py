"""Two changes of an LM iteration's schedule that change no arithmetic:
* the fork: the image sums and the after-linearization control of the
  previous linearization run on a second stream beside the point Schur and
  the key-pair assembly (plans of 300k keys or more; GBA_FORK=1 forks these
  small test plans too, GBA_ONE_STREAM=1 keeps one stream);
* the candidate's Jacobian records are formed by the candidate cost kernel
  into the other parity's buffer and become current when the step is
  accepted (GBA_SEPARATE_LINEARIZE=1 relinearizes in its own launch after
  the accept).
Each gives the same bits, reports and stop reasons as the other schedule,
also when problems stop early (small gradient or step) while the next
iteration's point Schur already ran for them, when steps are rejected (the
current records must survive a rejected candidate), with PCG and with free
cameras."""
import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

# (environment of the first run, of the second run)
SWITCHES = [("GBA_FORK", "GBA_ONE_STREAM"), (None, "GBA_SEPARATE_LINEARIZE")]


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def _both(gba, monkeypatch, env, scenes, opt):
    first, second = env
    if first:
        monkeypatch.setenv(first, "1")
    xs, reps = gba.solve_batch(scenes, opt)
    if first:
        monkeypatch.delenv(first)
    monkeypatch.setenv(second, "1")
    xo, repo = gba.solve_batch(scenes, opt)
    monkeypatch.delenv(second)
    for a, b, ra, rb in zip(xs, xo, reps, repo):
        np.testing.assert_array_equal(a, b)
        assert ra.final_cost == rb.final_cost
        assert (ra.iterations, ra.accepted, ra.rejected, ra.stop_reason, ra.status) == \
               (rb.iterations, rb.accepted, rb.rejected, rb.stop_reason, rb.status)
    return reps


@pytest.mark.parametrize("env", SWITCHES)
@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_same_bits_dense(gba, monkeypatch, env, precision):
    scenes = [synthetic.ring_scene(num_images=10, num_points=800, obs_range=(3, 8), seed=s) for s in (1, 2)]
    scenes.append(synthetic.grid_scene(num_images=30, num_points=3000, seed=4))
    _both(gba, monkeypatch, env, scenes, abi.make_options(max_iterations=8, eps1=0.0, eps2=0.0,
                                                          precision=precision))


@pytest.mark.parametrize("env", SWITCHES)
@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_same_bits_with_rejected_steps(gba, monkeypatch, env, precision):
    """Twelve iterations without stopping tests: past convergence the
    candidates are rejected (about half of the steps)."""
    s = synthetic.ring_scene(num_images=8, num_points=400, seed=3)
    reps = _both(gba, monkeypatch, env, [s], abi.make_options(max_iterations=12, eps1=0.0, eps2=0.0,
                                                              precision=precision))
    assert reps[0].rejected > 0 and reps[0].accepted > 0
    # alone (one-problem dense plan: the dataflow factorization) as well
    if env[0]:
        monkeypatch.setenv(env[0], "1")
    x1, r1 = gba.solve(s, abi.make_options(max_iterations=12, eps1=0.0, eps2=0.0, precision=precision))
    if env[0]:
        monkeypatch.delenv(env[0])
    monkeypatch.setenv(env[1], "1")
    x2, r2 = gba.solve(s, abi.make_options(max_iterations=12, eps1=0.0, eps2=0.0, precision=precision))
    monkeypatch.delenv(env[1])
    np.testing.assert_array_equal(x1, x2)
    assert (r1.accepted, r1.rejected) == (r2.accepted, r2.rejected)


@pytest.mark.parametrize("env", SWITCHES)
def test_same_bits_early_stops(gba, monkeypatch, env):
    """Stopping tests on: the problems stop at different iterations."""
    scenes = [synthetic.ring_scene(num_images=8, num_points=500, seed=s) for s in (3, 4, 5)]
    reps = _both(gba, monkeypatch, env, scenes, abi.make_options(max_iterations=40, eps1=1e-6, eps2=1e-10,
                                                                 precision=abi.PRECISION_FP64))
    assert any(r.iterations < 40 for r in reps)


@pytest.mark.parametrize("env", SWITCHES)
def test_same_bits_pcg(gba, monkeypatch, env):
    scenes = [synthetic.walk_scene(num_images=50, num_points=3000, mean_obs=8.0, seed=s,
                                   outlier_fraction=0.01, max_track=30) for s in (6, 7)]
    _both(gba, monkeypatch, env, scenes, abi.make_options(max_iterations=5, eps1=0.0, eps2=0.0,
                                                          precision=abi.PRECISION_MIXED,
                                                          linear_solver=abi.LINEAR_PCG,
                                                          loss=abi.LOSS_HUBER, huber_delta=1.0))


@pytest.mark.parametrize("env", SWITCHES)
@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_same_bits_free_cameras(gba, monkeypatch, env, precision):
    s = synthetic.full_model_scene(seed=3, num_images=8, num_points=300, num_cameras=2, fix_mask=0)
    _both(gba, monkeypatch, env, [s], abi.make_options(max_iterations=6, eps1=0.0, eps2=0.0,
                                                       precision=precision))
