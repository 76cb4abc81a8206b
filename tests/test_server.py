"""The continuous-batching server (gba_server_*): a request's result is the
same bits alone and in any micro-batch, cancelled requests report
GBA_ERR_CANCELLED, requests above the memory budget are refused at submit,
and the admission estimate bounds the bytes a plan really holds."""
import time

import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic


def _requests(n, seed=21):
    return synthetic.window_batch(num_windows=n, seed=seed, images_range=(5, 16),
                                  points_range=(200, 1500))


def test_estimate_is_host_only_and_monotone():
    from hs_sfm_gb300 import gba
    small, big = _requests(1, seed=1)[0], synthetic.ring_scene(num_images=30, num_points=4000)
    e_small = gba.estimate_device_bytes(small, abi.PRECISION_MIXED)
    e_big = gba.estimate_device_bytes(big, abi.PRECISION_MIXED)
    assert 0 < e_small < e_big
    assert gba.estimate_device_bytes(big, abi.PRECISION_MIXED) < \
        gba.estimate_device_bytes(big, abi.PRECISION_FP64)


def test_server_without_device_fails_loudly():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is visible")
    from hs_sfm_gb300 import gba
    with pytest.raises(gba.GbaError) as e:
        gba.Server()
    assert e.value.status == abi.GBA_ERR_NO_DEVICE


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_results_identical_alone_and_batched(precision):
    from hs_sfm_gb300 import gba
    scenes = _requests(7)
    opt = dict(max_iterations=15, precision=precision)
    alone = [gba.solve(s, abi.make_options(**opt))[0] for s in scenes]
    cfg = gba.default_server_config(**opt)
    cfg.max_batch, cfg.max_in_flight = 3, 2
    with gba.Server(cfg) as srv:
        tickets = [srv.submit(s) for s in scenes]
        out = [srv.wait(t, timeout_ms=120_000) for t in tickets]
        st = srv.stats()
    for (x, rep), xa in zip(out, alone):
        assert rep.status == abi.GBA_OK
        assert np.array_equal(x, xa)
        assert 0.0 <= rep.queue_ms <= rep.latency_ms
    assert st["completed"] == len(scenes)
    assert st["batches_launched"] >= 3
    assert st["admitted_bytes"] == 0 and st["in_flight_requests"] == 0


@pytest.mark.gpu
def test_cancel_queued_request():
    from hs_sfm_gb300 import gba
    scenes = _requests(6, seed=5)
    cfg = gba.default_server_config(max_iterations=30, precision=abi.PRECISION_MIXED)
    cfg.max_batch, cfg.max_in_flight = 1, 1
    with gba.Server(cfg) as srv:
        tickets = [srv.submit(s) for s in scenes]
        srv.cancel(tickets[-1])
        for t in tickets[:-1]:
            x, rep = srv.wait(t, timeout_ms=120_000)
            assert rep.status == abi.GBA_OK
        with pytest.raises(gba.GbaError) as e:
            srv.wait(tickets[-1], timeout_ms=120_000)
        assert e.value.status == abi.GBA_ERR_CANCELLED
        st = srv.stats()
    assert st["cancelled"] == 1 and st["completed"] == len(scenes) - 1


@pytest.mark.gpu
def test_refuse_over_budget_and_poll():
    from hs_sfm_gb300 import gba
    scenes = _requests(2, seed=9)
    need = max(gba.estimate_device_bytes(s, abi.PRECISION_MIXED) for s in scenes)
    cfg = gba.default_server_config(max_iterations=10, precision=abi.PRECISION_MIXED)
    cfg.memory_budget_bytes = need
    with gba.Server(cfg) as srv:
        big = synthetic.ring_scene(num_images=40, num_points=20_000)
        with pytest.raises(gba.GbaError) as e:
            srv.submit(big)
        assert e.value.status == abi.GBA_ERR_BUSY
        # both fit alone, not together: they run one after the other
        tickets = [srv.submit(s) for s in scenes]
        deadline = time.time() + 120
        results = {}
        while len(results) < len(tickets) and time.time() < deadline:
            for t in tickets:
                if t not in results:
                    r = srv.poll(t)
                    if r is not None:
                        results[t] = r
            time.sleep(0.002)
        st = srv.stats()
    assert len(results) == 2
    assert st["refused"] == 1 and st["completed"] == 2
    with pytest.raises(gba.GbaError):
        srv_bad = gba.Server(cfg)
        try:
            srv_bad.poll(12345)
        finally:
            srv_bad.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [abi.PRECISION_MIXED, abi.PRECISION_FP64])
def test_estimate_bounds_plan_bytes(precision):
    from hs_sfm_gb300 import gba
    extra = [synthetic.ring_scene(num_images=60, num_points=5000),
             synthetic.full_model_scene(seed=3, num_images=20, num_points=2000, num_cameras=2,
                                        obs_per_point=4),               # free cameras
             synthetic.full_model_scene(seed=4, num_images=12, num_points=1500, num_cameras=12,
                                        obs_per_point=4),               # a camera per image
             synthetic.gcp_scene(seed=5, num_images=20, num_points=3000, num_gcps=10)]
    for s in _requests(4, seed=13) + extra:
        est = gba.estimate_device_bytes(s, precision)
        p = gba.Plan(s, abi.make_options(precision=precision, max_iterations=1))
        real = p.device_bytes()
        p.close()
        assert real <= est <= 3 * real + (2 << 20), (s.name, real, est)



@pytest.mark.gpu
def test_server_free_cameras_and_priors_match_alone():
    # requests of the extended models through the server equal their solo solves
    from hs_sfm_gb300 import gba
    scenes = [synthetic.full_model_scene(seed=21, num_images=10, num_points=400, obs_per_point=4),
              synthetic.gcp_scene(seed=22, num_images=10, num_points=500, num_gcps=6),
              synthetic.full_model_scene(seed=23, num_images=8, num_points=300,
                                         fix_mask=abi.FIX_CAMERAS, obs_per_point=4)]
    cfg = gba.default_server_config(precision=abi.PRECISION_FP64)
    cfg.solve.max_iterations = 8
    cfg.solve.eps1 = 0.0
    cfg.solve.eps2 = 0.0
    with gba.Server(cfg) as srv:
        tickets = [srv.submit(s) for s in scenes]
        outs = [srv.wait(t) for t in tickets]
    for s, (x, rep) in zip(scenes, outs):
        x1, r1 = gba.solve(s, cfg.solve)
        assert rep.status == abi.GBA_OK
        assert rep.final_cost == r1.final_cost and np.array_equal(x, x1)


@pytest.mark.gpu
def test_server_fixed_groups_and_pcg_free_cameras_match_alone():
    """Requests with points or images fixed (every mask but all three) and a
    PCG solve with free cameras through the server: each result has the
    caller's x layout and equals the same request solved alone."""
    from helpers import ALL_FIX_MASKS
    from hs_sfm_gb300 import gba
    scenes = [synthetic.full_model_scene(seed=40 + m, num_images=8, num_points=250, fix_mask=m,
                                         obs_per_point=4) for m in ALL_FIX_MASKS]
    cfg = gba.default_server_config(precision=abi.PRECISION_FP64)
    cfg.solve.max_iterations = 6
    cfg.solve.eps1 = 0.0
    cfg.solve.eps2 = 0.0
    with gba.Server(cfg) as srv:
        tickets = [srv.submit(s) for s in scenes]
        outs = [srv.wait(t) for t in tickets]
    for s, (x, rep) in zip(scenes, outs):
        assert len(x) == abi.x_size(s)
        x1, r1 = gba.solve(s, cfg.solve)
        assert rep.status == abi.GBA_OK
        assert rep.final_cost == r1.final_cost and np.array_equal(x, x1)
    free = synthetic.full_model_scene(seed=50, num_images=10, num_points=400, obs_per_point=4)
    cfg.solve.linear_solver = abi.LINEAR_PCG
    cfg.solve.pcg_max_iterations = 300
    cfg.solve.pcg_relative_tolerance = 1e-12
    with gba.Server(cfg) as srv:
        x, rep = srv.wait(srv.submit(free))
    x1, r1 = gba.solve(free, cfg.solve)
    assert rep.status == abi.GBA_OK and rep.pcg_iterations > 0
    assert rep.final_cost == r1.final_cost and np.array_equal(x, x1)
