"""Bounded device waits: the dataflow factorization's CTAs poll flags other
CTAs publish; with the poll limit lowered (GBA_DF_SPIN_LIMIT) a CTA that finds
nothing ready gives up, raises the abort word, and the solve returns
GBA_ERR_TIMEOUT -- no fault, no hang, and the device stays usable.  The
cluster backward solve's warps wait on per-step mbarriers; with one step's
delta withheld (GBA_SOLVE_DROP_STEP) and the limit lowered
(GBA_SOLVE_SPIN_LIMIT) the waits run out and the solve reports the same."""
import os
import subprocess
import sys

import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys
sys.path.insert(0, {root!r})
from hs_sfm_gb300 import abi, gba, synthetic
s = synthetic.ring_scene(num_images=40, num_points=1500, seed=4)
try:
    gba.solve(s, abi.make_options(max_iterations=3))
    print("STATUS 0")
except gba.GbaError as e:
    print("STATUS", e.status)
s2 = synthetic.ring_scene(num_images=6, num_points=200, seed=5)
x, r = gba.solve(s2, abi.make_options(max_iterations=3, shared_device=1))
print("AFTER", r.status)
"""


def test_dataflow_wait_times_out_and_device_stays_usable():
    env = dict(os.environ, GBA_DF_SPIN_LIMIT="1")
    out = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = dict(l.split(" ", 1) for l in out.stdout.strip().splitlines())
    assert int(lines["STATUS"]) == abi.GBA_ERR_TIMEOUT
    assert int(lines["AFTER"]) == abi.GBA_OK


def test_default_limit_is_not_reached():
    from hs_sfm_gb300 import gba
    s = synthetic.ring_scene(num_images=40, num_points=1500, seed=4)
    x, rep = gba.solve(s, abi.make_options(max_iterations=3))
    assert rep.status == abi.GBA_OK and np.all(np.isfinite(x))


CHILD_SOLVE = r"""
import os, sys
sys.path.insert(0, {root!r})
from hs_sfm_gb300 import abi, gba, synthetic
# 48 images: a 288-unknown system of 9 tile rows, solved by the cluster kernel
s = synthetic.ring_scene(num_images=48, num_points=2000, obs_per_point=4, seed=6)
try:
    gba.solve(s, abi.make_options(max_iterations=3))
    print("STATUS 0")
except gba.GbaError as e:
    print("STATUS", e.status)
os.environ.pop("GBA_SOLVE_SPIN_LIMIT")
os.environ.pop("GBA_SOLVE_DROP_STEP")
x, r = gba.solve(s, abi.make_options(max_iterations=3))
print("AFTER", r.status)
"""


def test_solve_wait_times_out_and_device_stays_usable():
    # the owner of tile row 4 never sends its delta: every other warp's
    # bounded wait for it runs out, the solve reports GBA_ERR_TIMEOUT, and the
    # next solve in the same process is normal
    env = dict(os.environ, GBA_SOLVE_SPIN_LIMIT="2000", GBA_SOLVE_DROP_STEP="4")
    out = subprocess.run([sys.executable, "-c", CHILD_SOLVE.format(root=ROOT)], env=env,
                         capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    lines = dict(l.split(" ", 1) for l in out.stdout.strip().splitlines())
    assert int(lines["STATUS"]) == abi.GBA_ERR_TIMEOUT
    assert int(lines["AFTER"]) == abi.GBA_OK
