"""Generates the golden fixtures under tests/golden/.

projection_fixture.json: image keys of the reference's known-answer
derivative fixture (unit_test/bundle_adjustment/
test_camera_shared_analytical_derivative.cpp:746-770, values copied as
numbers) and of 16 seeded random cases, computed by an implementation that is
independent of the oracle: scipy's Rotation.from_rotvec for the angle-axis
rotation, then the distortion and intrinsic formulas of
sfm_utility/radial_distortor.hpp:14-28, decentering_distortor.hpp:14-24 and
camera_shared_vector_function.hpp:731-744.

Run: python tests/golden/make_golden.py
"""
import json
import os

import numpy as np
from scipy.spatial.transform import Rotation

HERE = os.path.dirname(os.path.abspath(__file__))

# The reference fixture (test_camera_shared_analytical_derivative.cpp:746-770).
FIXTURE = {
    "point": [89.06332903711264, -254.7119654139254, 27.36102981725708],
    "rotation": [0.0461972342123952, -0.01398317345699249, -1.02689361003788],
    "translation": [228.8962690432249, 77.85673263411233, -476.5385356161123],
    "k": [-0.005049046200604883, 0.03129380429860988, -0.03079482096044222],
    "d": [-0.0005537654832018913, -0.0004987771776838148],
    "intrinsic": [4835.47665904517, 0.0, -42.4095312016, -31.699212823, 1.0],
}


def project(point, rotation, translation, k, d, intrinsic):
    pc = Rotation.from_rotvec(rotation).apply(point) + np.asarray(translation)
    x, y = pc[0] / pc[2], pc[1] / pc[2]
    r2 = x * x + y * y
    coeff = k[0] * r2 + k[1] * r2 ** 2 + k[2] * r2 ** 3
    dx = coeff * x + 2 * d[0] * x * y + d[1] * (r2 + 2 * x * x)
    dy = coeff * y + 2 * d[1] * x * y + d[0] * (r2 + 2 * y * y)
    nx, ny = x + dx, y + dy
    f, s, cx, cy, a = intrinsic
    return [f * nx + s * ny + cx, f * a * ny + cy], [x, y]


def main():
    cases = []
    f = FIXTURE
    key, nkey = project(f["point"], f["rotation"], f["translation"], f["k"], f["d"], f["intrinsic"])
    cases.append(dict(FIXTURE, key=key, normalized=nkey, name="reference_fixture"))
    rng = np.random.default_rng(12345)
    for i in range(16):
        rot = rng.normal(0, 1.0, 3)
        pt = rng.uniform(-2, 2, 3)
        tr = np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(6, 12)])
        k = rng.uniform(-0.1, 0.1, 3)
        d = rng.uniform(-1e-3, 1e-3, 2)
        intr = [rng.uniform(800, 1200), rng.uniform(-1, 1), rng.uniform(900, 1000),
                rng.uniform(500, 580), rng.uniform(0.95, 1.05)]
        key, nkey = project(pt, rot, tr, k, d, intr)
        cases.append(dict(point=pt.tolist(), rotation=rot.tolist(), translation=tr.tolist(),
                          k=k.tolist(), d=d.tolist(), intrinsic=intr, key=key, normalized=nkey,
                          name=f"random{i}"))
    with open(os.path.join(HERE, "projection_fixture.json"), "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py (scipy Rotation.from_rotvec)",
                   "cases": cases}, fh, indent=1)


if __name__ == "__main__":
    main()
