"""Scene builders shared by the tests."""
import json
import os

import numpy as np

from hs_sfm_gb300 import abi, synthetic

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

ALL_FIX_MASKS = [0, 1, 2, 3, 4, 5, 6]  # every combination but all-fixed


def fixture_cases():
    with open(os.path.join(GOLDEN, "projection_fixture.json")) as fh:
        return json.load(fh)["cases"]


def single_key_scene(case, mask):
    """One point, one image, one camera, everything free: x = [point,
    rotation, translation, camera] as in the reference's derivative test
    (test_camera_shared_analytical_derivative.cpp:566-731)."""
    cam = []
    if mask & abi.COMPUTE_RADIAL:
        cam += case["k"]
    if mask & abi.COMPUTE_DECENTERING:
        cam += case["d"]
    if mask & abi.COMPUTE_INTRINSIC:
        cam += case["intrinsic"]
    cameras = np.array(cam, dtype=np.float64).reshape(1, -1)
    points = np.array(case["point"], dtype=np.float64).reshape(1, 3)
    images = np.array(case["rotation"] + case["translation"], dtype=np.float64).reshape(1, 6)
    s = synthetic.Scene(name="single", points=points, images=images, cameras=cameras,
                        image_camera_map=np.zeros(1, np.int64),
                        feature_maps=np.array([[0, 0]], np.int64), intrinsic_mask=mask,
                        fix_mask=0, near_y=np.zeros(2), x0=None, x_true=None)
    x = np.concatenate([points.reshape(-1), images.reshape(-1), cameras.reshape(-1)])
    s.x0 = x
    s.x_true = x
    return s, x


def fix_scene(scene, fix_mask):
    """The same scene with another fix mask (x and the fixed blocks rebuilt
    from the truth; constraint targets recomputed)."""
    s = synthetic.full_model_scene(seed=7, fix_mask=fix_mask)
    return s


def full_scene(fix_mask, seed=7, **kw):
    return synthetic.full_model_scene(seed=seed, fix_mask=fix_mask, **kw)


def is_approx(a, b, prec):
    """Eigen's isApprox: ||a - b|| <= prec * min(||a||, ||b||)."""
    a, b = np.asarray(a), np.asarray(b)
    return np.linalg.norm(a - b) <= prec * min(np.linalg.norm(a), np.linalg.norm(b))


def abs_rel_ok(ref, val, threshold):
    """The reference's elementwise test: fail only when both the absolute and
    the relative error exceed the threshold
    (test_camera_shared_jacobian_matrix_calculator.cpp:121-160)."""
    ref, val = np.asarray(ref), np.asarray(val)
    err = np.abs(ref - val)
    rel = np.where(ref != 0, err / np.where(ref != 0, np.abs(ref), 1), err)
    return bool(np.all((err <= threshold) | (rel <= threshold))), float(err.max()), float(rel.max())
