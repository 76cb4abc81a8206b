"""Batched multi-view triangulation on the device against the oracle
(triangulate/multiple_view_dlt.hpp, multiple_view_levenberg_marquardt_optimizor.hpp,
multiple_view_maximum_likelihood_estimator.hpp; sfm_utility/projective_functions.hpp,
undistortor.hpp)."""
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


def test_noise_free_tracks_recover_the_points(gba):
    b = synthetic.triangulation_batch(seed=1, num_points=5000, noise=0.0)
    P, st = gba.triangulate(b)
    assert np.all(st == abi.GBA_OK)
    assert np.max(np.abs(P - b.points)) < 1e-9


def per_point_cost(b, Pts):
    k = np.diff(b.track_offsets)
    r = synthetic.project_views(b.intrinsics, b.extrinsics, b.track_views,
                                np.repeat(Pts, k, axis=0)) - b.track_keys
    return np.add.reduceat(np.sum(r * r, axis=1), b.track_offsets[:-1])


def assert_same_points(b, P, Pr):
    # The same DLT start and LM steps in FP64; the device contracts
    # multiply-adds, so a poorly conditioned track (two close views) can stop
    # one LM step apart along its flat direction: the points agree to 1e-6
    # and their reprojection costs to 1e-9 relative.
    assert np.max(np.abs(P - Pr)) < 1e-6
    c, cr = per_point_cost(b, P), per_point_cost(b, Pr)
    assert np.all(np.abs(c - cr) <= 1e-9 * cr + 1e-12)


@pytest.mark.parametrize("distortion", [False, True])
def test_matches_oracle(gba, distortion):
    b = synthetic.triangulation_batch(seed=2, num_points=4000, noise=0.5, distortion=distortion)
    opt = abi.make_options()
    P, st = gba.triangulate(b, opt)
    Pr, sr = oracle.triangulate(b, opt)
    assert np.array_equal(st, sr) and np.all(st == abi.GBA_OK)
    assert_same_points(b, P, Pr)


def test_dlt_only_matches_oracle(gba):
    b = synthetic.triangulation_batch(seed=3, num_points=2000, noise=1.0)
    opt = abi.make_options(max_iterations=0)
    P, _ = gba.triangulate(b, opt)
    Pr, _ = oracle.triangulate(b, opt)
    assert np.max(np.abs(P - Pr)) < 1e-8


def test_refinement_lowers_the_reprojection_cost(gba):
    b = synthetic.triangulation_batch(seed=4, num_points=3000, noise=1.0)
    P0, _ = gba.triangulate(b, abi.make_options(max_iterations=0))
    P, _ = gba.triangulate(b)
    c0, c1 = per_point_cost(b, P0), per_point_cost(b, P)
    assert np.all(c1 <= c0 * (1 + 1e-12) + 1e-12)
    assert c1.sum() < c0.sum()


def test_short_tracks_and_bad_views(gba):
    b = synthetic.triangulation_batch(seed=5, num_points=50, noise=0.5)
    # point 3 keeps one observation only: the reference returns -1 for it
    keep = np.ones(len(b.track_views), dtype=bool)
    s, e = b.track_offsets[3], b.track_offsets[4]
    keep[s + 1:e] = False
    k = np.diff(b.track_offsets).copy()
    k[3] = 1
    b.track_views = b.track_views[keep]
    b.track_keys = b.track_keys[keep]
    b.track_offsets = np.concatenate([[0], np.cumsum(k)]).astype(np.int64)
    P, st = gba.triangulate(b)
    Pr, sr = oracle.triangulate(b)
    assert st[3] == abi.GBA_ERR_INVALID and sr[3] == abi.GBA_ERR_INVALID
    assert np.all(np.delete(st, 3) == abi.GBA_OK)
    b.track_views = b.track_views.copy()
    b.track_views[0] = len(b.intrinsics)
    with pytest.raises(gba.GbaError) as e:
        gba.triangulate(b)
    assert e.value.status == abi.GBA_ERR_BAD_INDEX
