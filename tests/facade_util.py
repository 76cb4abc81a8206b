"""Builds tests/cpp/facade_solve.cpp against libgba.so and writes problems
in its input format."""
import os
import subprocess

import numpy as np

from hs_sfm_gb300 import build as gba_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_facade(out_dir):
    lib = gba_build.build()
    exe = os.path.join(out_dir, "facade_solve")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_solve.cpp"), "-o", exe,
                    "-L", os.path.dirname(lib), "-lgba", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True)
    return exe


def write_problem(path, scene, iters, mode=0):
    with open(path, "wb") as fh:
        np.array([scene.number_of_points, scene.number_of_images, scene.number_of_cameras,
                  scene.number_of_keys, scene.intrinsic_mask, iters, mode], np.int64).tofile(fh)
        np.ascontiguousarray(scene.feature_maps, np.int64).tofile(fh)
        np.ascontiguousarray(scene.image_camera_map, np.int64).tofile(fh)
        np.ascontiguousarray(scene.cameras, np.float64).tofile(fh)
        np.ascontiguousarray(scene.near_y, np.float64).tofile(fh)
        np.ascontiguousarray(scene.x0, np.float64).tofile(fh)
