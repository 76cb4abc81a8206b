"""The work-item sizes (gba_options.pair_item / image_item / key_item), the Z
layout and gba_autotune:
any item size gives the same model (costs within the parity tolerance of the
default split and of the FP64 oracle, a problem's bits the same alone and in
a batch with the same sizes), bad sizes are refused, and the tuner returns a
timed candidate from its search set."""
import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

OPT = dict(max_iterations=6, eps1=0.0, eps2=0.0)


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def test_item_sizes_keep_the_model(gba):
    s = synthetic.ring_scene(num_images=12, num_points=3000, obs_per_point=6, seed=41)
    x_ref, r_ref = gba.solve(s, abi.make_options(**OPT))
    for pi, ii, ki in ((32, 32, 64), (100, 7, 300), (4096, 2048, 4096)):
        x, r = gba.solve(s, abi.make_options(pair_item=pi, image_item=ii, key_item=ki, **OPT))
        assert r.status == abi.GBA_OK
        assert abs(r.final_cost - r_ref.final_cost) <= 1e-9 * r_ref.final_cost
        np.testing.assert_allclose(x, x_ref, rtol=0, atol=1e-7)
    _, _, rref = oracle.lm_solve(s, options=abi.make_options(**OPT))
    assert abs(r.final_cost - rref.final_cost) <= 1e-9 * rref.final_cost


def test_batch_equals_alone_with_item_sizes(gba):
    scenes = [synthetic.ring_scene(num_images=n, num_points=400 * n, obs_range=(3, 8), seed=50 + n)
              for n in (5, 9, 14)]
    opt = abi.make_options(precision=abi.PRECISION_MIXED, pair_item=128, image_item=64, key_item=320,
                           **OPT)
    xs, reps = gba.solve_batch(scenes, opt)
    for s, x, r in zip(scenes, xs, reps):
        x1, r1 = gba.solve(s, opt)
        assert np.array_equal(x, x1) and r.final_cost == r1.final_cost


def test_bad_item_sizes_are_refused(gba):
    s = synthetic.ring_scene(num_images=4, num_points=50, obs_per_point=3, seed=42)
    for kw in (dict(pair_item=-1), dict(image_item=-5), dict(pair_item=1 << 25), dict(key_item=-2),
               dict(key_item=1 << 25)):
        with pytest.raises(gba.GbaError) as e:
            gba.solve(s, abi.make_options(**kw, **OPT))
        assert e.value.status == abi.GBA_ERR_INVALID


def test_autotune_picks_a_timed_candidate(gba):
    scenes = [synthetic.ring_scene(num_images=n, num_points=1500 * n, obs_range=(3, 8), seed=60 + n)
              for n in (6, 12, 20, 30)]
    opt = abi.make_options(precision=abi.PRECISION_MIXED, max_iterations=10)
    t = gba.autotune(scenes, opt)
    assert t["candidates"] == 11   # ten item-size candidates, then the other Z layout
    assert t["pair_item"] in (256, 512, 1024, 2048, 4096)
    assert t["image_item"] in (256, 512, 1024)
    assert t["key_item"] in (256, 512, 1024, 2048)
    assert t["z_layout"] in (abi.Z_RECORDS, abi.Z_PLANES)
    assert 0 < t["ms_per_iteration"] <= t["default_ms_per_iteration"]
    # with the layout given, only the item sizes are searched
    fixed = gba.autotune(scenes[:1], abi.make_options(precision=abi.PRECISION_MIXED, max_iterations=10,
                                                      z_layout=abi.Z_RECORDS))
    assert fixed["candidates"] == 10 and fixed["z_layout"] == abi.Z_RECORDS
    tuned = abi.make_options(precision=abi.PRECISION_MIXED, max_iterations=10, eps1=0.0, eps2=0.0,
                             pair_item=t["pair_item"], image_item=t["image_item"],
                             key_item=t["key_item"], z_layout=t["z_layout"])
    xs, reps = gba.solve_batch(scenes, tuned)
    _, _, rref = oracle.lm_solve(scenes[0], options=abi.make_options(max_iterations=10, eps1=0.0,
                                                                      eps2=0.0))
    assert abs(reps[0].final_cost - rref.final_cost) <= 1e-6 * rref.final_cost
