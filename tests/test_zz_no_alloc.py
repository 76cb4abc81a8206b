"""gba_cost_noalloc: the cost of a problem already in device memory, computed
with no device allocation (for callers that cannot call cudaMalloc, e.g. a
plugin inside an application that owns every device allocation).  Its
result must match gba_cost, the allocating entry point, within the cost
tolerance of the parity tests (1e-12 relative), on two calls in a row.

This file is collected last so that a run stopping at the first failure has
already run every other test."""
import ctypes as C

import numpy as np
import pytest

from hs_sfm_gb300 import abi, synthetic

pytestmark = pytest.mark.gpu

COST_RTOL = 1e-12


class DeviceProblem(C.Structure):
    _fields_ = [("number_of_points", C.c_int32), ("number_of_images", C.c_int32),
                ("number_of_cameras", C.c_int32), ("number_of_keys", C.c_int32),
                ("key_image", C.c_void_p), ("key_point", C.c_void_p), ("keys", C.c_void_p),
                ("image_camera", C.c_void_p), ("cameras", C.c_void_p), ("points", C.c_void_p),
                ("images", C.c_void_p)]


def full_cameras(scene):
    out = np.tile(np.array([0, 0, 0, 0, 0, 1, 0, 0, 0, 1], np.float64), (scene.number_of_cameras, 1))
    o = 0
    if scene.intrinsic_mask & abi.COMPUTE_RADIAL:
        out[:, 0:3] = scene.cameras[:, 0:3]
        o = 3
    if scene.intrinsic_mask & abi.COMPUTE_DECENTERING:
        out[:, 3:5] = scene.cameras[:, o:o + 2]
        o += 2
    if scene.intrinsic_mask & abi.COMPUTE_INTRINSIC:
        out[:, 5:10] = scene.cameras[:, o:o + 5]
    return out


def upload(scene, x):
    import torch
    P = scene.number_of_points
    t = {
        "key_image": torch.tensor(scene.feature_maps[:, 0], dtype=torch.int32, device="cuda"),
        "key_point": torch.tensor(scene.feature_maps[:, 1], dtype=torch.int32, device="cuda"),
        "keys": torch.tensor(scene.near_y[:2 * scene.number_of_keys], dtype=torch.float64, device="cuda"),
        "image_camera": torch.tensor(scene.image_camera_map, dtype=torch.int32, device="cuda"),
        "cameras": torch.tensor(full_cameras(scene).reshape(-1), dtype=torch.float64, device="cuda"),
        "points": torch.tensor(x[:3 * P], dtype=torch.float64, device="cuda"),
        "images": torch.tensor(x[3 * P:], dtype=torch.float64, device="cuda"),
    }
    dp = DeviceProblem(P, scene.number_of_images, scene.number_of_cameras, scene.number_of_keys,
                       *[t[k].data_ptr() for k in ("key_image", "key_point", "keys", "image_camera",
                                                    "cameras", "points", "images")])
    return dp, t


def noalloc_cost(L, dp, loss, delta, out=None):
    import torch
    if out is None:
        out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = L.gba_cost_noalloc(C.byref(dp), loss, delta, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
    assert st == 0, st
    torch.cuda.synchronize()
    return float(out.item())


@pytest.fixture(scope="module")
def L():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from hs_sfm_gb300 import gba
    lib = gba.lib()
    lib.gba_cost_noalloc.argtypes = [C.POINTER(DeviceProblem), C.c_int32, C.c_double,
                                     C.c_void_p, C.c_void_p]
    return lib


@pytest.mark.parametrize("loss", [abi.LOSS_TRIVIAL, abi.LOSS_HUBER])
def test_noalloc_cost_matches_allocating_entry_point(L, loss):
    from hs_sfm_gb300 import gba
    s = synthetic.ring_scene(num_images=24, num_points=3000, obs_per_point=5, seed=31,
                             mask=abi.COMPUTE_RADIAL | abi.COMPUTE_INTRINSIC)
    s.cameras = s.cameras.copy()
    s.cameras[0, 0:2] = [0.03, -0.02]
    opt = abi.make_options(loss=loss, huber_delta=1.0)
    ref = gba.cost(s, s.x0, options=opt)
    dp, keep = upload(s, s.x0)
    first = noalloc_cost(L, dp, loss, 1.0)
    second = noalloc_cost(L, dp, loss, 1.0)
    assert abs(first - ref) <= COST_RTOL * ref, (first, ref)
    assert abs(second - ref) <= COST_RTOL * ref, (second, ref)
    # a different problem through the same scratch, then the first again
    s2 = synthetic.ring_scene(num_images=7, num_points=500, obs_per_point=3, seed=32)
    dp2, keep2 = upload(s2, s2.x0)
    ref2 = gba.cost(s2, s2.x0, options=opt)
    assert abs(noalloc_cost(L, dp2, loss, 1.0) - ref2) <= COST_RTOL * ref2
    assert abs(noalloc_cost(L, dp, loss, 1.0) - ref) <= COST_RTOL * ref


def test_noalloc_rejects_oversized_problem(L):
    import torch
    s = synthetic.ring_scene(num_images=4, num_points=40, obs_per_point=2, seed=33)
    dp, keep = upload(s, s.x0)
    dp.number_of_images = 16385   # one past GBA_NOALLOC_MAX_IMAGES
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = L.gba_cost_noalloc(C.byref(dp), 0, 1.0, C.c_void_p(out.data_ptr()), C.c_void_p(0))
    assert st == abi.GBA_ERR_INVALID


def test_noalloc_allocates_nothing(L):
    """The point of the entry point: after a first call on the device, calls
    leave the device's free memory exactly as they found it."""
    import torch
    s = synthetic.ring_scene(num_images=12, num_points=2000, obs_per_point=4, seed=34)
    dp, keep = upload(s, s.x0)
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    noalloc_cost(L, dp, abi.LOSS_TRIVIAL, 1.0, out)   # first call: loads the kernels
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    values = [noalloc_cost(L, dp, abi.LOSS_HUBER if i % 2 else abi.LOSS_TRIVIAL, 1.0, out)
              for i in range(8)]
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before, (free_before, free_after)
    assert values[0] == values[2] and values[1] == values[3]


def test_noalloc_rejects_missing_images_before_any_launch(L):
    """Zero keys but images present: the rotation pass would read images, so a
    NULL images pointer is refused on the host."""
    import torch
    s = synthetic.ring_scene(num_images=4, num_points=40, obs_per_point=2, seed=35)
    dp, keep = upload(s, s.x0)
    dp.number_of_keys = 0
    dp.images = None
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    before = L.gba_kernel_launch_count()
    st = L.gba_cost_noalloc(C.byref(dp), 0, 1.0, C.c_void_p(out.data_ptr()), C.c_void_p(0))
    assert st == abi.GBA_ERR_INVALID
    assert L.gba_kernel_launch_count() == before
    # zero keys with the images present is a valid call with cost 0
    dp2, keep2 = upload(s, s.x0)
    dp2.number_of_keys = 0
    assert noalloc_cost(L, dp2, abi.LOSS_TRIVIAL, 1.0) == 0.0


def test_noalloc_out_of_range_ids_give_nan_without_fault(L):
    """Ids are checked on the device: a key pointing past the points (or an
    image pointing past the cameras) is skipped and the cost is NaN; the next
    call on the same scratch is normal again."""
    import math
    import torch
    s = synthetic.ring_scene(num_images=6, num_points=300, obs_per_point=3, seed=36)
    dp, keep = upload(s, s.x0)
    good = noalloc_cost(L, dp, abi.LOSS_TRIVIAL, 1.0)
    bad_pt = keep["key_point"].clone()
    bad_pt[5] = s.number_of_points + 1000
    dp_bad = DeviceProblem(dp.number_of_points, dp.number_of_images, dp.number_of_cameras,
                           dp.number_of_keys, dp.key_image, bad_pt.data_ptr(), dp.keys,
                           dp.image_camera, dp.cameras, dp.points, dp.images)
    assert math.isnan(noalloc_cost(L, dp_bad, abi.LOSS_TRIVIAL, 1.0))
    bad_cam = keep["image_camera"].clone()
    bad_cam[0] = -1
    dp_cam = DeviceProblem(dp.number_of_points, dp.number_of_images, dp.number_of_cameras,
                           dp.number_of_keys, dp.key_image, dp.key_point, dp.keys,
                           bad_cam.data_ptr(), dp.cameras, dp.points, dp.images)
    assert math.isnan(noalloc_cost(L, dp_cam, abi.LOSS_TRIVIAL, 1.0))
    assert noalloc_cost(L, dp, abi.LOSS_TRIVIAL, 1.0) == good
    torch.cuda.synchronize()
