"""Edge cases of the device path against the oracle: empty and degenerate
problems, ragged batches, images without keys, single-key points, and the
dense solver's size limit (2,048 reduced-system images)."""
import numpy as np
import pytest

import oracle
from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

OPT = dict(max_iterations=10, eps1=0.0, eps2=0.0)


@pytest.fixture(scope="module")
def gba():
    from hs_sfm_gb300 import gba as g
    g.lib()
    return g


def subset(s, keep_keys):
    """The scene with only the keys keep_keys (mask), observations and weights in step."""
    t = synthetic.Scene(**{**s.__dict__})
    t.feature_maps = s.feature_maps[keep_keys]
    K = s.number_of_keys
    y = s.near_y[:2 * K].reshape(-1, 2)[keep_keys].reshape(-1)
    t.near_y = np.concatenate([y, s.near_y[2 * K:]])
    return t


def test_problem_without_keys(gba):
    s = synthetic.ring_scene(num_images=4, num_points=30, obs_per_point=2, seed=2)
    e = subset(s, np.zeros(s.number_of_keys, dtype=bool))
    x, rep = gba.solve(e, abi.make_options(**OPT))
    err, x_ref, rref = oracle.lm_solve(e, options=abi.make_options(**OPT))
    assert rep.status == abi.GBA_OK and err == 0
    assert rep.final_cost == 0.0 == rref.final_cost
    np.testing.assert_array_equal(x, e.x0)   # nothing to move: g = 0 stops at once
    assert rep.stop_reason == rref.stop_reason


def test_images_without_keys_and_single_key_points(gba):
    s = synthetic.ring_scene(num_images=8, num_points=400, obs_per_point=3, seed=3)
    fm = s.feature_maps
    keep = fm[:, 0] != 5                       # image 5 loses every key
    first = np.r_[True, fm[1:, 1] != fm[:-1, 1]]
    lone = np.isin(fm[:, 1], np.arange(0, 400, 7))
    keep &= ~lone | first                      # every 7th point keeps one key only
    t = subset(s, keep)
    assert not np.any(t.feature_maps[:, 0] == 5)
    for prec in (abi.PRECISION_FP64, abi.PRECISION_MIXED):
        x, rep = gba.solve(t, abi.make_options(precision=prec, **OPT))
        err, x_ref, rref = oracle.lm_solve(t, options=abi.make_options(**OPT))
        assert rep.status == abi.GBA_OK and err == 0
        assert abs(rep.final_cost - rref.final_cost) <= 1e-6 * rref.final_cost
        # the keyless image does not move (its gradient is zero, its block mu I)
        i5 = 3 * t.number_of_points + 6 * 5
        np.testing.assert_array_equal(x[i5:i5 + 6], t.x0[i5:i5 + 6])


def test_ragged_batch_with_empty_and_tiny_problems(gba):
    s0 = synthetic.ring_scene(num_images=3, num_points=20, obs_per_point=2, seed=4)
    empty = subset(s0, np.zeros(s0.number_of_keys, dtype=bool))
    tiny = synthetic.ring_scene(num_images=2, num_points=5, obs_per_point=2, seed=5)
    big = synthetic.ring_scene(num_images=40, num_points=3000, obs_per_point=6, seed=6)
    mid = synthetic.full_model_scene(seed=7, num_images=9, num_points=300, obs_per_point=4)
    scenes = [tiny, empty, big, mid, empty, tiny]
    opt = abi.make_options(**OPT)
    xs, reps = gba.solve_batch(scenes, opt)
    for s, x, r in zip(scenes, xs, reps):
        x1, r1 = gba.solve(s, opt)
        assert r.status == abi.GBA_OK
        assert np.array_equal(x, x1) and r.final_cost == r1.final_cost
        _, _, rref = oracle.lm_solve(s, options=opt)
        # (the tiny problems are underdetermined: their cost falls to rounding level)
        assert abs(r.final_cost - rref.final_cost) <= 1e-9 * rref.final_cost + 1e-12


def test_dense_size_limit(gba):
    # 2,048 images is the dense solver's largest problem (a 12,288-unknown
    # reduced system); one more is refused, and PCG takes it
    s = synthetic.ring_scene(num_images=2048, num_points=20000, obs_per_point=3, seed=8)
    opt = dict(max_iterations=2, eps1=0.0, eps2=0.0)
    x, rep = gba.solve(s, abi.make_options(precision=abi.PRECISION_MIXED, **opt))
    x64, rep64 = gba.solve(s, abi.make_options(precision=abi.PRECISION_FP64, **opt))
    assert rep.status == abi.GBA_OK and rep64.status == abi.GBA_OK
    assert rep.final_cost < rep.initial_cost
    assert abs(rep.final_cost - rep64.final_cost) <= 1e-6 * rep64.final_cost
    s2 = synthetic.ring_scene(num_images=2049, num_points=2049, obs_per_point=2, seed=9)
    with pytest.raises(gba.GbaError) as e:
        gba.solve(s2, abi.make_options(**opt))
    assert e.value.status == abi.GBA_ERR_UNSUPPORTED
    _, rp = gba.solve(s2, abi.make_options(linear_solver=abi.LINEAR_PCG, **opt))
    assert rp.status == abi.GBA_OK


def test_solve_batch_into_keeps_x0_and_matches_in_place(gba):
    # gba_solve_batch_into reads x0 and writes separate outputs: the same
    # bits as the in-place gba_solve_batch, and the callers' x0 untouched
    import ctypes as C
    scenes = [synthetic.ring_scene(num_images=n, num_points=200 * n, obs_per_point=3, seed=70 + n)
              for n in (4, 7)]
    keep = [s.x0.copy() for s in scenes]
    opt = abi.make_options(**OPT)
    xs, reps = gba.solve_batch(scenes, opt)              # through gba_solve_batch_into
    for s, k in zip(scenes, keep):
        np.testing.assert_array_equal(s.x0, k)
    L = gba.lib()
    cps = [abi.CProblem(s) for s in scenes]
    arr = (abi.Problem * len(cps))(*[c.problem for c in cps])
    ys = [np.ascontiguousarray(s.near_y, dtype=np.float64) for s in scenes]
    xi = [np.ascontiguousarray(s.x0, dtype=np.float64).copy() for s in scenes]
    yp = (C.POINTER(C.c_double) * 2)(*[abi.dptr(y) for y in ys])
    xp = (C.POINTER(C.c_double) * 2)(*[abi.dptr(x) for x in xi])
    reps2 = (abi.Report * 2)()
    assert L.gba_solve_batch(arr, yp, 2, C.byref(opt), xp, reps2) == abi.GBA_OK
    for a, b, r, r2 in zip(xs, xi, reps, reps2):
        np.testing.assert_array_equal(a, b)
        assert r.final_cost == r2.final_cost
