"""Builds tests/cpp/facade_solve.cpp against libgba.so and writes problems
in its input format."""
import os
import subprocess

import numpy as np

from hs_sfm_gb300 import build as gba_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_facade(out_dir, driver="facade_solve"):
    lib = gba_build.build()
    exe = os.path.join(out_dir, driver)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", driver + ".cpp"), "-o", exe,
                    "-L", os.path.dirname(lib), "-lgba", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True)
    return exe


def gcp_naive_layout(scene):
    """A point-prior scene in the GCP-constrained model's layout: points
    renumbered so the control points come last (in prior order), x as
    [cameras 6C][points 3P].  Returns (perm, x0_naive) with perm[new] = old."""
    P = scene.number_of_points
    pri = list(scene.point_priors)
    rest = [p for p in range(P) if p not in set(pri)]
    perm = np.array(rest + pri, dtype=np.int64)
    P3 = 3 * P
    pts = scene.x0[:P3].reshape(-1, 3)[perm]
    x0 = np.concatenate([scene.x0[P3:], pts.reshape(-1)])
    return perm, x0


def write_gcp_problem(path, scene, iters):
    perm, x0 = gcp_naive_layout(scene)
    inv = np.empty_like(perm)
    inv[perm] = np.arange(len(perm))
    fm = np.ascontiguousarray(scene.feature_maps, np.int64).copy()
    fm[:, 1] = inv[fm[:, 1]]
    G = len(scene.point_priors)
    with open(path, "wb") as fh:
        np.array([scene.number_of_images, scene.number_of_points, scene.number_of_keys, G, iters],
                 np.int64).tofile(fh)
        fm.tofile(fh)
        np.ascontiguousarray(scene.near_y, np.float64).tofile(fh)
        np.ascontiguousarray(scene.key_covariance_inverse, np.float64).tofile(fh)
        np.ascontiguousarray(scene.prior_information, np.float64).tofile(fh)
        np.ascontiguousarray(x0, np.float64).tofile(fh)
    return perm


def write_problem(path, scene, iters, mode=0):
    with open(path, "wb") as fh:
        np.array([scene.number_of_points, scene.number_of_images, scene.number_of_cameras,
                  scene.number_of_keys, scene.intrinsic_mask, iters, mode], np.int64).tofile(fh)
        np.ascontiguousarray(scene.feature_maps, np.int64).tofile(fh)
        np.ascontiguousarray(scene.image_camera_map, np.int64).tofile(fh)
        np.ascontiguousarray(scene.cameras, np.float64).tofile(fh)
        np.ascontiguousarray(scene.near_y, np.float64).tofile(fh)
        np.ascontiguousarray(scene.x0, np.float64).tofile(fh)
        if mode == 3:   # the fixed points follow x0
            np.ascontiguousarray(scene.points, np.float64).tofile(fh)


def write_triangulation(path, b):
    """A synthetic.TriangulationBatch in tests/cpp/triangulate_solve.cpp's input format."""
    n = len(b.track_offsets) - 1
    with open(path, "wb") as fh:
        np.array([len(b.intrinsics), n, len(b.track_views)], np.int64).tofile(fh)
        np.ascontiguousarray(b.intrinsics, np.float64).tofile(fh)
        np.ascontiguousarray(b.extrinsics, np.float64).tofile(fh)
        np.ascontiguousarray(b.track_offsets, np.int64).tofile(fh)
        np.ascontiguousarray(b.track_views, np.int64).tofile(fh)
        np.ascontiguousarray(b.track_keys, np.float64).tofile(fh)
