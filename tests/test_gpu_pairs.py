"""The device's block and pair build (pair counts per image pair, block
numbering, enumeration and a stable radix sort by block) against the
host's: plans without free cameras build their blocks and key-pair list on
the device unless GBA_HOST_PAIRS is set, and both must give the same solve,
bit for bit -- one radix pass (fewer than 256 blocks), two and three passes
(more than 65,536 blocks), the dense and the PCG solver, FP64 and mixed,
single-key points, keyless images, ragged batches with empty problems."""
import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

OPT = dict(max_iterations=4, eps1=0.0, eps2=0.0)


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def both(gba, monkeypatch, scene, opt):
    monkeypatch.delenv("GBA_HOST_PAIRS", raising=False)
    x_dev, r_dev = gba.solve(scene, opt)
    monkeypatch.setenv("GBA_HOST_PAIRS", "1")
    x_host, r_host = gba.solve(scene, opt)
    monkeypatch.delenv("GBA_HOST_PAIRS", raising=False)
    assert r_dev.status == abi.GBA_OK and r_host.status == abi.GBA_OK
    np.testing.assert_array_equal(x_dev, x_host)
    assert r_dev.final_cost == r_host.final_cost
    assert r_dev.iterations == r_host.iterations
    return r_dev


@pytest.mark.parametrize("prec", [abi.PRECISION_FP64, abi.PRECISION_MIXED])
def test_one_pass_dense(gba, monkeypatch, prec):
    s = synthetic.ring_scene(num_images=12, num_points=2000, obs_per_point=5, seed=21)
    r = both(gba, monkeypatch, s, abi.make_options(precision=prec, **OPT))
    assert r.final_cost < r.initial_cost


@pytest.mark.parametrize("solver", [abi.LINEAR_DENSE_CHOLESKY, abi.LINEAR_PCG])
def test_two_passes_grid(gba, monkeypatch, solver):
    s = synthetic.grid_scene(num_images=120, num_points=20_000, seed=22)
    both(gba, monkeypatch, s, abi.make_options(precision=abi.PRECISION_MIXED,
                                                 linear_solver=solver, **OPT))


def test_three_passes_walk(gba, monkeypatch):
    # long tracks over 2,000 images: about 60 neighbours per image, more than
    # 65,536 blocks, so the block ids need three 8-bit digits
    s = synthetic.walk_scene(num_images=2000, num_points=60_000, mean_obs=20.0, seed=23)
    both(gba, monkeypatch, s, abi.make_options(precision=abi.PRECISION_MIXED,
                                                 linear_solver=abi.LINEAR_PCG,
                                                 max_iterations=2, eps1=0.0, eps2=0.0))


def test_single_key_points_and_keyless_images(gba, monkeypatch):
    s = synthetic.ring_scene(num_images=9, num_points=600, obs_per_point=3, seed=24)
    fm = s.feature_maps
    keep = fm[:, 0] != 4
    first = np.r_[True, fm[1:, 1] != fm[:-1, 1]]
    keep &= ~np.isin(fm[:, 1], np.arange(0, 600, 5)) | first
    t = synthetic.Scene(**{**s.__dict__})
    t.feature_maps = fm[keep]
    K = s.number_of_keys
    y = s.near_y[:2 * K].reshape(-1, 2)[keep].reshape(-1)
    t.near_y = np.concatenate([y, s.near_y[2 * K:]])
    both(gba, monkeypatch, t, abi.make_options(**OPT))


def test_presorted_keys_take_the_same_path(gba):
    # keys already by point then image skip the host sort; any other order
    # is sorted into the same layout, so the solves agree bit for bit
    s = synthetic.grid_scene(num_images=40, num_points=5000, seed=25)
    fm = s.feature_maps
    assert np.all(np.diff(fm[:, 1]) >= 0)
    perm = np.random.default_rng(25).permutation(len(fm))
    t = synthetic.Scene(**{**s.__dict__})
    t.feature_maps = fm[perm]
    K = s.number_of_keys
    y = s.near_y[:2 * K].reshape(-1, 2)[perm].reshape(-1)
    t.near_y = np.concatenate([y, s.near_y[2 * K:]])
    opt = abi.make_options(precision=abi.PRECISION_MIXED, **OPT)
    x0, r0 = gba.solve(s, opt)
    x1, r1 = gba.solve(t, opt)
    np.testing.assert_array_equal(x0, x1)
    assert r0.final_cost == r1.final_cost


@pytest.mark.parametrize("solver", [abi.LINEAR_DENSE_CHOLESKY, abi.LINEAR_PCG])
def test_batch_blocks_on_device(gba, monkeypatch, solver):
    # a ragged batch (empty, tiny and larger problems): the problems' code
    # ranges follow each other, the device's blocks and pairs are the host's
    s0 = synthetic.ring_scene(num_images=3, num_points=20, obs_per_point=2, seed=26)
    empty = synthetic.Scene(**{**s0.__dict__})
    empty.feature_maps = s0.feature_maps[:0]
    empty.near_y = s0.near_y[2 * s0.number_of_keys:]
    scenes = [synthetic.ring_scene(num_images=2, num_points=5, obs_per_point=2, seed=27), empty,
              synthetic.ring_scene(num_images=30, num_points=3000, obs_range=(3, 8), seed=28),
              synthetic.grid_scene(num_images=40, num_points=4000, seed=29), empty,
              synthetic.ring_scene(num_images=12, num_points=800, obs_per_point=5, seed=30)]
    opt = abi.make_options(precision=abi.PRECISION_MIXED, linear_solver=solver, **OPT)
    monkeypatch.delenv("GBA_HOST_PAIRS", raising=False)
    xs_dev, reps_dev = gba.solve_batch(scenes, opt)
    monkeypatch.setenv("GBA_HOST_PAIRS", "1")
    xs_host, reps_host = gba.solve_batch(scenes, opt)
    monkeypatch.delenv("GBA_HOST_PAIRS", raising=False)
    for xd, xh, rd, rh in zip(xs_dev, xs_host, reps_dev, reps_host):
        assert rd.status == abi.GBA_OK and rh.status == abi.GBA_OK
        np.testing.assert_array_equal(xd, xh)
        assert rd.final_cost == rh.final_cost
