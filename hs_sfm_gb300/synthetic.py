"""Seeded synthetic bundle-adjustment scenes.

The reference ships its own scene generators (include/hs_sfm/synthetic/ and
bundle_adjustment/camera_shared_synthetic_data_generator.hpp:47-847) driven by
an external, unseeded RNG; these are new seeded generators with the shapes,
sizes and value distributions of the five benchmark workloads:

  ring   -- cameras evenly on a circle looking at the origin, points in a
            cube, each point seen by its k nearest cameras (10 cameras /
            1,000 points / 5 per point; also each window of the 512-window
            batch and each serving request);
  grid   -- 200 cameras on a jittered grid looking down on a
            [-20,20]^2 x [-2,2] slab of 100,000 points, each point seen by
            4-12 cameras drawn uniformly among those that see it, radial
            distortion k1, k2 ~ U(-0.1, 0.1);
  walk   -- 2,000 cameras on a random walk (step 1.0) over 1,000,000 points,
            geometric track lengths with mean 10 and 1% outlier keys.

Keys are projected with the reference model, perturbed by N(0, 1 px) noise
and rounded to float32 (so a float32 copy of the observations is exact).  The
initial x perturbs rotations by Exp(N(0, 0.01)) * R, translations by
N(0, 0.05) and points by N(0, 0.05).
"""
from __future__ import annotations

import dataclasses

import numpy as np

COMPUTE_RADIAL = 1
COMPUTE_DECENTERING = 2
COMPUTE_INTRINSIC = 4
FIX_POINTS = 1
FIX_IMAGES = 2
FIX_CAMERAS = 4


def params_per_camera(mask: int) -> int:
    return (3 if mask & COMPUTE_RADIAL else 0) + (2 if mask & COMPUTE_DECENTERING else 0) + \
        (5 if mask & COMPUTE_INTRINSIC else 0)


# ---------------------------------------------------------------------------
# Rotation helpers (angle-axis <-> matrix), vectorised.
# ---------------------------------------------------------------------------
def rotvec_to_matrix(r: np.ndarray) -> np.ndarray:
    r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
    theta = np.linalg.norm(r, axis=1)
    out = np.tile(np.eye(3), (len(r), 1, 1))
    nz = theta > 0
    k = np.zeros_like(r)
    k[nz] = r[nz] / theta[nz, None]
    K = np.zeros((len(r), 3, 3))
    K[:, 0, 1], K[:, 0, 2] = -k[:, 2], k[:, 1]
    K[:, 1, 0], K[:, 1, 2] = k[:, 2], -k[:, 0]
    K[:, 2, 0], K[:, 2, 1] = -k[:, 1], k[:, 0]
    s, c = np.sin(theta)[:, None, None], np.cos(theta)[:, None, None]
    out = out + s * K + (1 - c) * (K @ K)
    return out


def matrix_to_rotvec(R: np.ndarray) -> np.ndarray:
    from scipy.spatial.transform import Rotation
    return Rotation.from_matrix(np.asarray(R).reshape(-1, 3, 3)).as_rotvec()


def look_at(center: np.ndarray, target: np.ndarray, up: np.ndarray) -> np.ndarray:
    """World->camera rotation with +z toward target and image y down."""
    z = target - center
    z = z / np.linalg.norm(z, axis=-1, keepdims=True)
    y = -up - np.sum(-up * z, axis=-1, keepdims=True) * z
    y = y / np.linalg.norm(y, axis=-1, keepdims=True)
    x = np.cross(y, z)
    return np.stack([x, y, z], axis=-2)


# ---------------------------------------------------------------------------
# The projection model of camera_shared_vector_function.hpp:634-744,
# vectorised (FP64).  images [N,6], points [N,3], cameras [N,cps].
# ---------------------------------------------------------------------------
def project(points, images, cameras, mask):
    points = np.asarray(points, np.float64)
    R = rotvec_to_matrix(images[:, :3])
    pc = np.einsum('nij,nj->ni', R, points) + images[:, 3:6]
    n = pc[:, :2] / pc[:, 2:3]
    off = 0
    delta = np.zeros_like(n)
    if mask & COMPUTE_RADIAL:
        k1, k2, k3 = cameras[:, 0], cameras[:, 1], cameras[:, 2]
        r2 = n[:, 0] ** 2 + n[:, 1] ** 2
        coeff = k1 * r2 + k2 * r2 ** 2 + k3 * r2 ** 3
        delta += coeff[:, None] * n
        off += 3
    if mask & COMPUTE_DECENTERING:
        d1, d2 = cameras[:, off], cameras[:, off + 1]
        x, y = n[:, 0], n[:, 1]
        r2 = x * x + y * y
        delta[:, 0] += 2 * d1 * x * y + d2 * (r2 + 2 * x * x)
        delta[:, 1] += 2 * d2 * x * y + d1 * (r2 + 2 * y * y)
        off += 2
    n = n + delta
    if mask & COMPUTE_INTRINSIC:
        f, s, cx, cy, a = (cameras[:, off + j] for j in range(5))
        u = f * n[:, 0] + s * n[:, 1] + cx
        v = f * a * n[:, 1] + cy
        return np.stack([u, v], axis=1), pc[:, 2]
    return n, pc[:, 2]


def _distort_intrinsic(n, cam, mask):
    """Distortion and intrinsics of camera_shared_vector_function.hpp:645-685
    applied to normalized keys n [..., 2] of a single camera."""
    off = 0
    x, y = n[..., 0], n[..., 1]
    r2 = x * x + y * y
    dx = np.zeros_like(x)
    dy = np.zeros_like(y)
    if mask & COMPUTE_RADIAL:
        coeff = cam[0] * r2 + cam[1] * r2 ** 2 + cam[2] * r2 ** 3
        dx, dy = dx + coeff * x, dy + coeff * y
        off += 3
    if mask & COMPUTE_DECENTERING:
        d1, d2 = cam[off], cam[off + 1]
        dx = dx + 2 * d1 * x * y + d2 * (r2 + 2 * x * x)
        dy = dy + 2 * d2 * x * y + d1 * (r2 + 2 * y * y)
        off += 2
    x, y = x + dx, y + dy
    if mask & COMPUTE_INTRINSIC:
        f, sk, cx, cy, a = cam[off:off + 5]
        return np.stack([f * x + sk * y + cx, f * a * y + cy], axis=-1)
    return np.stack([x, y], axis=-1)


# ---------------------------------------------------------------------------
# Scene container.
# ---------------------------------------------------------------------------
@dataclasses.dataclass
class Scene:
    name: str
    points: np.ndarray          # [P,3] truth
    images: np.ndarray          # [I,6] truth (r, t)
    cameras: np.ndarray         # [C,cps]
    image_camera_map: np.ndarray  # [I] int64
    feature_maps: np.ndarray    # [K,2] int64 (image_id, point_id)
    intrinsic_mask: int
    fix_mask: int
    near_y: np.ndarray          # [y_size] observed keys (+ constraint targets)
    x0: np.ndarray              # [x_size] initial guess
    x_true: np.ndarray          # [x_size]
    outlier: np.ndarray | None = None   # [K] bool
    point_constraints: list | None = None   # [(point_id, mask)]
    image_constraints: list | None = None   # [(image_id, mask)]
    camera_constraints: list | None = None  # [(camera_id, radial, decentering, intrinsic)]
    key_covariance_inverse: np.ndarray | None = None  # [K,2,2]
    constraint_weights: np.ndarray | None = None
    point_priors: list | None = None             # [point_id] (ground control points)
    prior_information: np.ndarray | None = None  # [n,3,3] inverse covariances

    @property
    def number_of_points(self):
        return int(self.points.shape[0])

    @property
    def number_of_images(self):
        return int(self.images.shape[0])

    @property
    def number_of_cameras(self):
        return int(self.cameras.shape[0])

    @property
    def number_of_keys(self):
        return int(self.feature_maps.shape[0])


def _x_of(points, images, cameras, fix_mask):
    parts = []
    if not fix_mask & FIX_POINTS:
        parts.append(points.reshape(-1))
    if not fix_mask & FIX_IMAGES:
        parts.append(images.reshape(-1))
    if not fix_mask & FIX_CAMERAS:
        parts.append(cameras.reshape(-1))
    return np.concatenate(parts) if parts else np.zeros(0)


def _perturb(rng, points, images, rot_sigma=0.01, t_sigma=0.05, p_sigma=0.05):
    R = rotvec_to_matrix(images[:, :3])
    dR = rotvec_to_matrix(rng.normal(0.0, rot_sigma, size=(len(images), 3)))
    r0 = matrix_to_rotvec(dR @ R)
    t0 = images[:, 3:] + rng.normal(0.0, t_sigma, size=(len(images), 3))
    p0 = points + rng.normal(0.0, p_sigma, size=points.shape)
    return p0, np.concatenate([r0, t0], axis=1)


def project_keys(points, images, cameras, image_camera_map, feature_maps, mask):
    """Keys of every (image, point) pair of feature_maps, one rotation matrix
    per image."""
    Rm = rotvec_to_matrix(images[:, :3])
    im, pt = feature_maps[:, 0], feature_maps[:, 1]
    pc = np.einsum('nij,nj->ni', Rm[im], points[pt]) + images[im, 3:]
    n = pc[:, :2] / pc[:, 2:3]
    cams = cameras[image_camera_map[im]]
    if len(cameras) == 1:
        return _distort_intrinsic(n, cameras[0], mask)
    out = np.empty_like(n)
    for c in range(len(cameras)):
        sel = image_camera_map[im] == c
        out[sel] = _distort_intrinsic(n[sel], cameras[c], mask)
    del cams
    return out


def _finish(name, rng, points, images, cameras, icm, fm, mask, fix_mask,
            noise=1.0, outlier_fraction=0.0, width=1920.0, height=1080.0):
    P = len(points)
    keys = project_keys(points, images, cameras, icm, fm, mask)
    obs = keys + rng.normal(0.0, noise, size=keys.shape)
    outlier = None
    if outlier_fraction > 0:
        outlier = rng.random(len(fm)) < outlier_fraction
        n_out = int(outlier.sum())
        obs[outlier, 0] = rng.uniform(0.0, width, n_out)
        obs[outlier, 1] = rng.uniform(0.0, height, n_out)
    near_y = obs.astype(np.float32).astype(np.float64).reshape(-1)
    p0, i0 = _perturb(rng, points, images)
    x0 = _x_of(p0, i0, cameras, fix_mask)
    xt = _x_of(points, images, cameras, fix_mask)
    del P
    return Scene(name=name, points=points, images=images, cameras=cameras,
                 image_camera_map=icm.astype(np.int64), feature_maps=fm.astype(np.int64),
                 intrinsic_mask=mask, fix_mask=fix_mask, near_y=near_y, x0=x0, x_true=xt,
                 outlier=outlier)


def default_intrinsics(mask, rng=None, k_range=0.0):
    cam = []
    if mask & COMPUTE_RADIAL:
        if rng is not None and k_range > 0:
            cam += [rng.uniform(-k_range, k_range), rng.uniform(-k_range, k_range), 0.0]
        else:
            cam += [0.0, 0.0, 0.0]
    if mask & COMPUTE_DECENTERING:
        cam += [0.0, 0.0]
    if mask & COMPUTE_INTRINSIC:
        cam += [1000.0, 0.0, 960.0, 540.0, 1.0]
    return np.array(cam, dtype=np.float64)


def ring_scene(num_images=10, num_points=1000, obs_per_point=5, seed=0, scale=1.0,
               obs_range=None, mask=COMPUTE_INTRINSIC, fix_mask=FIX_CAMERAS,
               name="ring"):
    """Cameras evenly on a circle of radius 10*scale in the world XY plane
    looking at the origin with +Z up; points uniform in [-2,2]^3 * scale;
    each point seen by its obs_per_point nearest cameras (or a per-point
    count drawn from obs_range=(lo, hi) inclusive)."""
    rng = np.random.default_rng(seed)
    phi = 2 * np.pi * np.arange(num_images) / num_images
    centers = np.stack([10 * scale * np.cos(phi), 10 * scale * np.sin(phi),
                        np.zeros(num_images)], axis=1)
    R = look_at(centers, np.zeros((num_images, 3)), np.array([0.0, 0.0, 1.0]))
    r = matrix_to_rotvec(R)
    t = -np.einsum('nij,nj->ni', R, centers)
    images = np.concatenate([r, t], axis=1)
    points = rng.uniform(-2 * scale, 2 * scale, size=(num_points, 3))
    d = np.linalg.norm(points[:, None, :] - centers[None, :, :], axis=2)
    order = np.argsort(d, axis=1, kind='stable')
    if obs_range is None:
        k = np.full(num_points, min(obs_per_point, num_images))
    else:
        k = rng.integers(obs_range[0], obs_range[1] + 1, size=num_points)
        k = np.minimum(k, num_images)
    rows = np.repeat(np.arange(num_points), k)
    cols = np.arange(len(rows)) - np.repeat(np.cumsum(k) - k, k)
    img = order[rows, cols]
    fm = np.stack([img, rows], axis=1)
    cameras = default_intrinsics(mask)[None, :]
    icm = np.zeros(num_images, dtype=np.int64)
    return _finish(name, rng, points, images, cameras, icm, fm, mask, fix_mask)


def grid_scene(num_images=200, num_points=100_000, seed=1, height=12.0,
               obs_range=(4, 12), mask=COMPUTE_RADIAL | COMPUTE_INTRINSIC,
               fix_mask=FIX_CAMERAS, name="grid"):
    """Cameras on a jittered grid at `height` looking down on a
    [-20,20]^2 x [-2,2] slab; per point a count in obs_range drawn uniformly
    among the cameras whose image contains the point."""
    rng = np.random.default_rng(seed)
    nx = int(round(np.sqrt(num_images * 2)))
    ny = max(1, num_images // nx)
    while nx * ny < num_images:
        ny += 1
    gx, gy = np.meshgrid(np.linspace(-19, 19, nx), np.linspace(-18, 18, ny), indexing='ij')
    centers = np.stack([gx.reshape(-1), gy.reshape(-1), np.full(nx * ny, height)], axis=1)
    centers = centers[:num_images] + np.concatenate(
        [rng.uniform(-0.5, 0.5, size=(num_images, 2)), rng.uniform(-0.3, 0.3, size=(num_images, 1))],
        axis=1)
    base = np.array([[1.0, 0, 0], [0, -1.0, 0], [0, 0, -1.0]])
    jit = rotvec_to_matrix(rng.normal(0, 0.02, size=(num_images, 3)))
    R = jit @ base
    r = matrix_to_rotvec(R)
    t = -np.einsum('nij,nj->ni', R, centers)
    images = np.concatenate([r, t], axis=1)
    cameras = default_intrinsics(mask, rng, 0.1)[None, :]
    icm = np.zeros(num_images, dtype=np.int64)
    points = np.stack([rng.uniform(-20, 20, num_points), rng.uniform(-20, 20, num_points),
                       rng.uniform(-2, 2, num_points)], axis=1)
    want = rng.integers(obs_range[0], obs_range[1] + 1, size=num_points)
    Rm = rotvec_to_matrix(images[:, :3])
    rows_all, cols_all = [], []
    chunk = 10_000
    for s in range(0, num_points, chunk):
        e = min(num_points, s + chunk)
        Pn = e - s
        pc = np.einsum('pj,cij->pci', points[s:e], Rm) + images[None, :, 3:]
        depth = pc[..., 2]
        keys = _distort_intrinsic(pc[..., :2] / pc[..., 2:3], cameras[0], mask)
        vis = (depth > 0.1) & (keys[..., 0] > 0) & (keys[..., 0] < 1920) & \
              (keys[..., 1] > 0) & (keys[..., 1] < 1080)
        pr = rng.random((Pn, num_images))
        pr[~vis] = 2.0
        order = np.argsort(pr, axis=1)
        k = np.minimum(want[s:e], vis.sum(axis=1))
        k[k < 2] = 0
        take = np.arange(num_images)[None, :] < k[:, None]
        rows_all.append(np.repeat(np.arange(s, e), k))
        cols_all.append(order[take])
    rows = np.concatenate(rows_all)
    cols = np.concatenate(cols_all)
    o = np.lexsort((cols, rows))
    rows, cols = rows[o], cols[o]
    fm = np.stack([cols, rows], axis=1)
    # points without two observations are dropped (reindexed)
    used = np.unique(rows)
    remap = -np.ones(num_points, dtype=np.int64)
    remap[used] = np.arange(len(used))
    points = points[used]
    fm[:, 1] = remap[fm[:, 1]]
    return _finish(name, rng, points, images, cameras, icm, fm, mask, fix_mask)


def walk_scene(num_images=2000, num_points=1_000_000, mean_obs=10.0, seed=2, height=15.0,
               outlier_fraction=0.01, max_track=60, mask=COMPUTE_INTRINSIC,
               fix_mask=FIX_CAMERAS, name="walk"):
    """Cameras along a random walk (unit steps in XY) at `height` looking
    down; each point seen by a run of consecutive cameras whose length is
    geometric with mean `mean_obs`; 1% of keys replaced by outliers."""
    rng = np.random.default_rng(seed)
    ang = rng.uniform(0, 2 * np.pi, num_images)
    steps = np.stack([np.cos(ang), np.sin(ang)], axis=1)
    xy = np.cumsum(steps, axis=0)
    centers = np.concatenate([xy, np.full((num_images, 1), height)], axis=1)
    base = np.array([[1.0, 0, 0], [0, -1.0, 0], [0, 0, -1.0]])
    R = rotvec_to_matrix(rng.normal(0, 0.02, size=(num_images, 3))) @ base
    r = matrix_to_rotvec(R)
    t = -np.einsum('nij,nj->ni', R, centers)
    images = np.concatenate([r, t], axis=1)
    cameras = default_intrinsics(mask)[None, :]
    icm = np.zeros(num_images, dtype=np.int64)
    k = 1 + rng.geometric(1.0 / (mean_obs - 1.0), size=num_points)
    k = np.minimum(k, min(max_track, num_images))
    start = rng.integers(0, num_images - k + 1)
    # point near the mean of its cameras' centres
    cs = np.concatenate([np.zeros((1, 2)), np.cumsum(xy, axis=0)], axis=0)
    mean_xy = (cs[start + k] - cs[start]) / k[:, None]
    points = np.concatenate([mean_xy + rng.normal(0, 1.5, size=(num_points, 2)),
                             rng.uniform(-2, 2, size=(num_points, 1))], axis=1)
    rows = np.repeat(np.arange(num_points), k)
    offs = np.arange(len(rows)) - np.repeat(np.cumsum(k) - k, k)
    cols = np.repeat(start, k) + offs
    keys, depth = project(points[rows], images[cols], cameras[icm[cols]], mask)
    vis = (depth > 0.1) & (keys[:, 0] > -200) & (keys[:, 0] < 2120) & (keys[:, 1] > -200) & (keys[:, 1] < 1280)
    rows, cols = rows[vis], cols[vis]
    cnt = np.bincount(rows, minlength=num_points)
    keep_pt = cnt >= 2
    keep = keep_pt[rows]
    rows, cols = rows[keep], cols[keep]
    remap = -np.ones(num_points, dtype=np.int64)
    remap[keep_pt] = np.arange(int(keep_pt.sum()))
    points = points[keep_pt]
    fm = np.stack([cols, remap[rows]], axis=1)
    return _finish(name, rng, points, images, cameras, icm, fm, mask, fix_mask,
                   outlier_fraction=outlier_fraction)


def window_batch(num_windows=512, seed=3, images_range=(5, 40), points_range=(500, 20_000),
                 obs_range=(3, 8)):
    """The 512-window local-BA batch: ring scenes with their own seed and
    scale, I ~ U{5..40}, P ~ U{500..20000}, 3-8 keys per point."""
    rng = np.random.default_rng(seed)
    out = []
    for w in range(num_windows):
        I = int(rng.integers(images_range[0], images_range[1] + 1))
        P = int(rng.integers(points_range[0], points_range[1] + 1))
        scale = float(rng.uniform(0.5, 2.0))
        out.append(ring_scene(num_images=I, num_points=P, obs_range=obs_range,
                              seed=int(rng.integers(0, 2**31 - 1)), scale=scale,
                              name=f"window{w}"))
    return out


def request_sizes(num, seed=4, median_images=20, median_points=5000, sigma=0.5,
                  max_images=300, max_points=200_000):
    """Log-normal request sizes for the serving stream."""
    rng = np.random.default_rng(seed)
    I = np.clip(np.round(median_images * np.exp(rng.normal(0, sigma, num))), 5, max_images).astype(int)
    P = np.clip(np.round(median_points * np.exp(rng.normal(0, sigma, num))), 200, max_points).astype(int)
    return I, P


def config(n: int, **kw):
    """The benchmark workloads by index: 0 ring 10/1000/5, 1 grid 200/100k,
    2 walk 2000/1M, 3 the 512-window batch (list of scenes)."""
    if n == 0:
        return ring_scene(num_images=10, num_points=1000, obs_per_point=5, seed=0, name="cfg0", **kw)
    if n == 1:
        return grid_scene(name="cfg1", **kw)
    if n == 2:
        return walk_scene(name="cfg2", **kw)
    if n == 3:
        return window_batch(**kw)
    raise ValueError(n)


# ---------------------------------------------------------------------------
# Small full-model scenes for the stage tests: several cameras, every
# intrinsic group, optional soft constraints and per-key covariances.
# ---------------------------------------------------------------------------
def gcp_scene(seed=0, num_images=10, num_points=500, num_gcps=8, obs_per_point=4,
              key_sigma=1e-3, gcp_sigma=0.02, name="gcp"):
    """The GCP-constrained model (ba_gcp_constrained_vector_function.hpp):
    normalized keys (no intrinsics: mask 0, one camera without parameters)
    of the ring geometry, key noise key_sigma with inverse covariance
    I / key_sigma^2, and num_gcps ground control points whose observed
    coordinates carry correlated noise of a random 3x3 covariance
    (scale gcp_sigma) with that covariance's inverse as their prior."""
    s = ring_scene(num_images=num_images, num_points=num_points, obs_per_point=obs_per_point,
                   seed=seed, mask=0, fix_mask=FIX_CAMERAS, name=name)
    rng = np.random.default_rng(seed + 7919)
    keys = project_keys(s.points, s.images, s.cameras, s.image_camera_map, s.feature_maps, 0)
    obs = (keys + rng.normal(0.0, key_sigma, keys.shape)).reshape(-1)
    gcps = np.sort(rng.choice(num_points, num_gcps, replace=False)).astype(np.int64)
    A = rng.normal(0.0, 0.4, size=(num_gcps, 3, 3))
    cov = gcp_sigma ** 2 * (np.einsum('nij,nkj->nik', A, A) + np.eye(3)[None])
    noise = np.einsum('nij,nj->ni', np.linalg.cholesky(cov), rng.normal(size=(num_gcps, 3)))
    s.near_y = np.concatenate([obs, (s.points[gcps] + noise).reshape(-1)])
    s.key_covariance_inverse = np.tile(np.eye(2) / key_sigma ** 2, (s.number_of_keys, 1, 1))
    s.point_priors = [int(v) for v in gcps]
    s.prior_information = np.linalg.inv(cov)
    return s


def full_model_scene(seed=0, num_images=6, num_points=60, num_cameras=2, fix_mask=0,
                     mask=COMPUTE_RADIAL | COMPUTE_DECENTERING | COMPUTE_INTRINSIC,
                     constraints=True, covariances=True, obs_per_point=3):
    rng = np.random.default_rng(seed)
    s = ring_scene(num_images=num_images, num_points=num_points, obs_per_point=obs_per_point,
                   seed=seed, mask=mask, fix_mask=fix_mask)
    cps = params_per_camera(mask)
    cams = []
    for c in range(num_cameras):
        cam = []
        if mask & COMPUTE_RADIAL:
            cam += list(rng.uniform(-0.05, 0.05, 3))
        if mask & COMPUTE_DECENTERING:
            cam += list(rng.uniform(-1e-3, 1e-3, 2))
        if mask & COMPUTE_INTRINSIC:
            cam += [float(rng.uniform(900, 1100)), float(rng.uniform(-1, 1)),
                    float(rng.uniform(940, 980)), float(rng.uniform(520, 560)),
                    float(rng.uniform(0.98, 1.02))]
        cams.append(cam)
    cameras = np.array(cams, dtype=np.float64).reshape(num_cameras, cps)
    icm = (np.arange(num_images) % num_cameras).astype(np.int64)
    keys, _ = project(s.points[s.feature_maps[:, 1]], s.images[s.feature_maps[:, 0]],
                      cameras[icm[s.feature_maps[:, 0]]], mask)
    obs = (keys + rng.normal(0, 1.0, keys.shape)).reshape(-1)
    pcs, ics, ccs = [], [], []
    if constraints:
        pcs = [(int(p), int(rng.integers(1, 8))) for p in rng.choice(num_points, 4, replace=False)]
        ics = [(int(i), int(rng.integers(1, 16))) for i in rng.choice(num_images, 2, replace=False)]
        ccs = []
        for c in range(num_cameras):
            rm = int(rng.integers(0, 8)) if mask & COMPUTE_RADIAL else 0
            dm = int(rng.integers(0, 4)) if mask & COMPUTE_DECENTERING else 0
            im = int(rng.integers(0, 32)) if mask & COMPUTE_INTRINSIC else 0
            ccs.append((c, rm, dm, im))
    p0, i0 = _perturb(rng, s.points, s.images)
    c0 = cameras * (1 + rng.normal(0, 1e-3, cameras.shape))
    x0 = _x_of(p0, i0, c0, fix_mask)
    xt = _x_of(s.points, s.images, cameras, fix_mask)
    scene = Scene(name="full", points=s.points, images=s.images, cameras=cameras,
                  image_camera_map=icm, feature_maps=s.feature_maps, intrinsic_mask=mask,
                  fix_mask=fix_mask, near_y=obs, x0=x0, x_true=xt,
                  point_constraints=pcs, image_constraints=ics, camera_constraints=ccs)
    # constraint targets = true values + noise; weights positive
    from . import abi
    ny = abi.y_size(scene)
    rows = abi.constraint_rows(scene)
    targets = []
    for (x_index_true, _) in rows:
        targets.append(xt[x_index_true] + rng.normal(0, 1e-2))
    scene.near_y = np.concatenate([obs, np.array(targets, dtype=np.float64)])
    assert len(scene.near_y) == ny
    if covariances:
        A = rng.normal(0, 0.3, size=(len(s.feature_maps), 2, 2))
        cov = np.einsum('kij,klj->kil', A, A) + np.eye(2)[None]
        scene.key_covariance_inverse = np.linalg.inv(cov)
    if rows:
        scene.constraint_weights = rng.uniform(0.5, 2.0, size=len(rows))
    return scene


@dataclasses.dataclass
class TriangulationBatch:
    """Views (CameraIntrinsicParams [f skew cx cy pixel_ratio k1 k2 k3 d1 d2],
    CameraExtrinsicParams [angle-axis world to camera, position]) and point
    tracks (offsets, view of each observation, observed keys)."""
    intrinsics: np.ndarray     # [V,10]
    extrinsics: np.ndarray     # [V,6]
    track_offsets: np.ndarray  # [n+1]
    track_views: np.ndarray    # [m]
    track_keys: np.ndarray     # [m,2]
    points: np.ndarray         # [n,3] truth


def project_views(intrinsics, extrinsics, views, X):
    """Keys of points X [m,3] in views [m] (sfm_utility/projective_functions.hpp:22-52)."""
    R = rotvec_to_matrix(extrinsics[views, :3])
    c = np.einsum('mij,mj->mi', R, X - extrinsics[views, 3:])
    x, y = c[:, 0] / c[:, 2], c[:, 1] / c[:, 2]
    K = intrinsics[views]
    f, s, cx, cy, a, k1, k2, k3, d1, d2 = K.T
    r2 = x * x + y * y
    coeff = k1 * r2 + k2 * r2 ** 2 + k3 * r2 ** 3
    ex = x + coeff * x + 2 * d1 * x * y + d2 * (r2 + 2 * x * x)
    ey = y + coeff * y + 2 * d2 * x * y + d1 * (r2 + 2 * y * y)
    return np.stack([f * ex + s * ey + cx, f * a * ey + cy], axis=1)


def triangulation_batch(seed=0, num_points=1000, num_views=20, views_range=(2, 8),
                        noise=0.5, distortion=True):
    """Views on a ring of radius 10 looking at the origin (each with its own
    intrinsics), points uniform in [-2,2]^3, each seen by k ~ U(views_range)
    views of the ring about 15 degrees apart from a random first one, keys
    with N(0, noise) pixel noise."""
    rng = np.random.default_rng(seed)
    phi = 2 * np.pi * np.arange(num_views) / num_views + rng.uniform(0, 0.1, num_views)
    centers = np.stack([10 * np.cos(phi), 10 * np.sin(phi), rng.uniform(-1, 1, num_views)], axis=1)
    R = look_at(centers, np.zeros((num_views, 3)), np.array([0.0, 0.0, 1.0]))
    extr = np.concatenate([matrix_to_rotvec(R), centers], axis=1)
    intr = np.zeros((num_views, 10))
    intr[:, 0] = rng.uniform(900, 1100, num_views)
    intr[:, 1] = rng.uniform(-1, 1, num_views)
    intr[:, 2] = rng.uniform(940, 980, num_views)
    intr[:, 3] = rng.uniform(520, 560, num_views)
    intr[:, 4] = rng.uniform(0.98, 1.02, num_views)
    if distortion:
        intr[:, 5:7] = rng.uniform(-0.05, 0.05, (num_views, 2))
        intr[:, 7] = rng.uniform(-0.01, 0.01, num_views)
        intr[:, 8:10] = rng.uniform(-1e-3, 1e-3, (num_views, 2))
    pts = rng.uniform(-2, 2, size=(num_points, 3))
    k = rng.integers(views_range[0], views_range[1] + 1, size=num_points)
    k = np.minimum(k, num_views)
    off = np.concatenate([[0], np.cumsum(k)]).astype(np.int64)
    start = rng.integers(0, num_views, size=num_points)
    pos = np.arange(off[-1]) - np.repeat(off[:-1], k)
    stride = max(1, num_views // 24)   # about 15 degrees between a track's views
    views = ((np.repeat(start, k) + stride * pos) % num_views).astype(np.int64)
    X = np.repeat(pts, k, axis=0)
    keys = project_views(intr, extr, views, X) + rng.normal(0, noise, (len(views), 2))
    return TriangulationBatch(intrinsics=intr, extrinsics=extr, track_offsets=off,
                              track_views=views, track_keys=keys, points=pts)
