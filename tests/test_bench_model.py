"""The measurement arithmetic of bench.py, on the CPU: the whole-iteration
speed of light (algorithmic bytes and FLOPs of one LM iteration against the
measured HBM and FP32 FMA roofs), the per-stage algorithmic bytes, and the
pair count the assembly's bytes use."""
import importlib.util
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_iteration_roofline_by_hand(bench):
    K, P, I, pairs, tsz = 801_039, 100_000, 200, 3_941_280, 4
    r = bench.iteration_roofline(K, P, I, pairs, 0.645, 6787.2, 77.9, tsz)
    n = 6 * I
    b = 40.0 * K + 168.0 * P + 120.0 * I + 3.0 * tsz * n * n
    f = 216.0 * K + 45.0 * P + 144.0 * K + 216.0 * pairs + n ** 3 / 3.0
    assert r["algorithmic_bytes"] == pytest.approx(b)
    assert r["algorithmic_flops"] == pytest.approx(f)
    t_sol = max(b / 6787.2e9, f / 77.9e12)
    assert r["speed_of_light_us"] == pytest.approx(1e6 * t_sol)
    assert r["frac"] == pytest.approx(t_sol / 0.645e-3)
    assert r["bound"] == "fp32"           # the grid's FLOP term dominates
    # without an FMA roof the bound is the bytes
    r2 = bench.iteration_roofline(K, P, I, pairs, 0.645, 6787.2, None, tsz)
    assert r2["bound"] == "hbm" and r2["speed_of_light_us"] == pytest.approx(1e6 * b / 6787.2e9)


def test_stage_bytes_scale_with_the_workload(bench):
    a = bench.stage_bytes(1000, 200, 10, 4000, 20, 4)
    b = bench.stage_bytes(2000, 400, 20, 8000, 40, 4)
    for k in a:
        assert b[k] == pytest.approx(2 * a[k])   # linear in every size
    d = bench.stage_bytes(1000, 200, 10, 4000, 20, 8)
    for k in ("linearize", "point_schur", "assemble"):
        assert d[k] > a[k]                          # FP64 records are larger


def test_pair_count_is_the_sum_of_k_k_plus_1_over_2(bench):
    class S:
        pass
    s = S()
    k = np.array([3, 1, 5, 2])
    s.feature_maps = np.stack([np.zeros(k.sum(), dtype=np.int64),
                               np.repeat(np.arange(len(k)), k)], axis=1)
    s.number_of_points = len(k)
    assert bench.pair_count(s) == int(np.sum(k * (k + 1) // 2))
