"""ctypes mirror of include/gba.h and conversion of problems to it.

A problem is any object with the attributes of
CameraSharedVectorFunction<double> (camera_shared_vector_function.hpp:746-763):
number_of_points/images/cameras, feature_maps [K,2] (image_id, point_id),
image_camera_map [I], intrinsic_mask, fix_mask, the fixed blocks, the three
constraint lists and, from CameraSharedYCovarianceInverse, per-key 2x2
inverse covariances and per-constraint weights.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# status codes (gba.h)
GBA_OK = 0
GBA_ERR = -1
GBA_ERR_INVALID = -2
GBA_ERR_BAD_INDEX = -3
GBA_ERR_DUPLICATE = -4
GBA_ERR_UNSUPPORTED = -5
GBA_ERR_NOT_SPD = -6
GBA_ERR_NAN = -7
GBA_ERR_OOM = -8
GBA_ERR_CUDA = -9
GBA_ERR_TIMEOUT = -10
GBA_ERR_NO_DEVICE = -11
GBA_ERR_BUSY = -12
GBA_ERR_CANCELLED = -13

COMPUTE_RADIAL = 1
COMPUTE_DECENTERING = 2
COMPUTE_INTRINSIC = 4
FIX_POINTS = 1
FIX_IMAGES = 2
FIX_CAMERAS = 4

PRECISION_FP64 = 0
PRECISION_MIXED = 1
LOSS_TRIVIAL = 0
LOSS_HUBER = 1
LINEAR_DENSE_CHOLESKY = 0
LINEAR_PCG = 1
Z_AUTO, Z_RECORDS, Z_PLANES = 0, 1, 2

NUM_STAGES = 12
STOP_MAX_ITERATIONS = 0
STOP_SMALL_GRADIENT = 1
STOP_SMALL_STEP = 2
STOP_ERROR = 3
STOP_SMALL_COST_CHANGE = 4
STAGE_NAMES = ["linearize", "point_schur", "assemble", "factor", "backsub", "cost",
               "control", "assemble_dense", "solve", "image_reduce", "image_prep", "reserved"]


class PointConstraint(C.Structure):
    _fields_ = [("point_id", C.c_int64), ("mask", C.c_uint32), ("pad_", C.c_uint32)]


class ImageConstraint(C.Structure):
    _fields_ = [("image_id", C.c_int64), ("mask", C.c_uint32), ("pad_", C.c_uint32)]


class CameraConstraint(C.Structure):
    _fields_ = [("camera_id", C.c_int64), ("radial_mask", C.c_uint32),
                ("decentering_mask", C.c_uint32), ("intrinsic_mask", C.c_uint32),
                ("pad_", C.c_uint32)]


_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)


class Problem(C.Structure):
    _fields_ = [
        ("number_of_points", C.c_int64), ("number_of_images", C.c_int64),
        ("number_of_cameras", C.c_int64), ("number_of_keys", C.c_int64),
        ("feature_maps", _i64p), ("image_camera_map", _i64p),
        ("intrinsic_computations_mask", C.c_uint32), ("fix_mask", C.c_uint32),
        ("fix_points", _dp), ("fix_images", _dp), ("fix_cameras", _dp),
        ("number_of_point_constraints", C.c_int64),
        ("point_constraints", C.POINTER(PointConstraint)),
        ("number_of_image_constraints", C.c_int64),
        ("image_constraints", C.POINTER(ImageConstraint)),
        ("number_of_camera_constraints", C.c_int64),
        ("camera_constraints", C.POINTER(CameraConstraint)),
        ("key_covariance_inverse", _dp), ("constraint_weights", _dp),
        ("number_of_point_priors", C.c_int64), ("point_prior_ids", _i64p),
        ("point_prior_information", _dp),
    ]


class Options(C.Structure):
    _fields_ = [
        ("max_iterations", C.c_int32), ("tau", C.c_double), ("eps1", C.c_double),
        ("eps2", C.c_double), ("precision", C.c_int32), ("loss", C.c_int32),
        ("huber_delta", C.c_double), ("linear_solver", C.c_int32),
        ("pcg_max_iterations", C.c_int32), ("pcg_relative_tolerance", C.c_double),
        ("use_cuda_graph", C.c_int32), ("profile", C.c_int32), ("device", C.c_int32),
        ("shared_device", C.c_int32), ("function_tolerance", C.c_double),
        ("pair_item", C.c_int32), ("image_item", C.c_int32), ("key_item", C.c_int32),
        ("z_layout", C.c_int32),
    ]


class Tuning(C.Structure):
    _fields_ = [("pair_item", C.c_int32), ("image_item", C.c_int32),
                ("ms_per_iteration", C.c_double), ("default_ms_per_iteration", C.c_double),
                ("candidates", C.c_int32), ("key_item", C.c_int32), ("z_layout", C.c_int32),
                ("reserved_", C.c_int32 * 1)]


class Report(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("stop_reason", C.c_int32), ("iterations", C.c_int32),
        ("accepted", C.c_int32), ("rejected", C.c_int32), ("factor_failures", C.c_int32),
        ("pcg_iterations", C.c_int32), ("pad_", C.c_int32),
        ("initial_cost", C.c_double), ("final_cost", C.c_double), ("final_rmse", C.c_double),
        ("final_mu", C.c_double), ("final_gradient_inf_norm", C.c_double),
        ("setup_ms", C.c_double), ("solve_ms", C.c_double),
        ("stage_ms", C.c_double * NUM_STAGES),
        ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
        ("queue_ms", C.c_double), ("latency_ms", C.c_double),
    ]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_
             if name not in ("pad_", "stage_ms")}
        d["stage_ms"] = list(self.stage_ms)
        return d


class PlanStructure(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "problems", "keys", "points", "images", "key_pairs", "pair_items", "blocks",
        "image_items", "camera_records", "max_reduced_size", "factor_schedule", "z_layout",
        "forked")] + [("reserved_", C.c_int64 * 1)]

    def as_dict(self):
        return {name: int(getattr(self, name)) for name, _ in self._fields_ if name != "reserved_"}


class ServerConfig(C.Structure):
    _fields_ = [("solve", Options), ("memory_budget_bytes", C.c_int64), ("max_batch", C.c_int32),
                ("max_in_flight", C.c_int32), ("reserved_", C.c_int32 * 6)]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "submitted", "completed", "cancelled", "refused", "queued", "in_flight_requests",
        "in_flight_batches", "batches_launched", "admitted_bytes", "budget_bytes")]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Triangulation(C.Structure):
    _fields_ = [("number_of_views", C.c_int64), ("intrinsics", _dp), ("extrinsics", _dp),
                ("number_of_points", C.c_int64), ("track_offsets", _i64p),
                ("track_views", _i64p), ("track_keys", _dp)]


class CTriangulation:
    """Contiguous copies of a triangulation batch and the gba_triangulation
    that points at them."""

    def __init__(self, t):
        self.keep = []

        def arr(a, dt, typ):
            a = np.ascontiguousarray(a, dtype=dt).reshape(-1)
            self.keep.append(a)
            return _ptr(a, typ)

        p = Triangulation()
        p.number_of_views = int(len(t.intrinsics))
        p.intrinsics = arr(t.intrinsics, np.float64, C.c_double)
        p.extrinsics = arr(t.extrinsics, np.float64, C.c_double)
        p.number_of_points = int(len(t.track_offsets) - 1)
        p.track_offsets = arr(t.track_offsets, np.int64, C.c_int64)
        p.track_views = arr(t.track_views, np.int64, C.c_int64)
        p.track_keys = arr(t.track_keys, np.float64, C.c_double)
        self.problem = p
        self.n = p.number_of_points

    @property
    def ref(self):
        return C.byref(self.problem)


def make_options(max_iterations=50, tau=1e-3, eps1=1e-8, eps2=1e-8, precision=PRECISION_FP64,
                 loss=LOSS_TRIVIAL, huber_delta=1.0, linear_solver=LINEAR_DENSE_CHOLESKY,
                 pcg_max_iterations=100, pcg_relative_tolerance=1e-6, use_cuda_graph=1,
                 profile=0, device=0, shared_device=0, function_tolerance=0.0,
                 pair_item=0, image_item=0, key_item=0, z_layout=0) -> Options:
    """Defaults of the reference's relative-pair test
    (test_camera_shared_relative_pair.cpp:976-979)."""
    o = Options()
    o.max_iterations = max_iterations
    o.tau, o.eps1, o.eps2 = tau, eps1, eps2
    o.precision, o.loss, o.huber_delta = precision, loss, huber_delta
    o.linear_solver = linear_solver
    o.pcg_max_iterations, o.pcg_relative_tolerance = pcg_max_iterations, pcg_relative_tolerance
    o.use_cuda_graph, o.profile, o.device = use_cuda_graph, profile, device
    o.shared_device = shared_device
    o.function_tolerance = function_tolerance
    o.pair_item, o.image_item, o.key_item = pair_item, image_item, key_item
    o.z_layout = z_layout
    return o


def params_per_camera(mask: int) -> int:
    return (3 if mask & COMPUTE_RADIAL else 0) + (2 if mask & COMPUTE_DECENTERING else 0) + \
        (5 if mask & COMPUTE_INTRINSIC else 0)


def x_size(s) -> int:
    cps = params_per_camera(s.intrinsic_mask)
    n = 0
    if not s.fix_mask & FIX_POINTS:
        n += 3 * s.number_of_points
    if not s.fix_mask & FIX_IMAGES:
        n += 6 * s.number_of_images
    if not s.fix_mask & FIX_CAMERAS:
        n += cps * s.number_of_cameras
    return n


def constraint_rows(s):
    """[(x_index, group)] for each constraint row in y order
    (camera_shared_vector_function.hpp:483-629)."""
    rows = []
    P, I = s.number_of_points, s.number_of_images
    cps = params_per_camera(s.intrinsic_mask)
    xi = 0 if s.fix_mask & FIX_POINTS else 3 * P
    xc = xi + (0 if s.fix_mask & FIX_IMAGES else 6 * I)
    if not s.fix_mask & FIX_POINTS:
        for pid, m in (s.point_constraints or []):
            for b in range(3):
                if m & (1 << b):
                    rows.append((3 * pid + b, 0))
    if not s.fix_mask & FIX_IMAGES:
        for iid, m in (s.image_constraints or []):
            if m & 1:
                rows += [(xi + 6 * iid + b, 1) for b in range(3)]
            for b in range(3):
                if m & (2 << b):
                    rows.append((xi + 6 * iid + 3 + b, 1))
    if not s.fix_mask & FIX_CAMERAS:
        for cid, rm, dm, im in (s.camera_constraints or []):
            off = xc + cps * cid
            for b in range(3):
                if rm & (1 << b):
                    rows.append((off + b, 2))
            if s.intrinsic_mask & COMPUTE_RADIAL:
                off += 3
            for b in range(2):
                if dm & (1 << b):
                    rows.append((off + b, 2))
            if s.intrinsic_mask & COMPUTE_DECENTERING:
                off += 2
            for b in range(5):
                if im & (1 << b):
                    rows.append((off + b, 2))
    return rows


def point_priors(s):
    """Point ids of the problem's priors (ground control points), or []."""
    return list(getattr(s, "point_priors", None) or [])


def y_size(s) -> int:
    """Keys, constraint rows, then 3 rows per point prior."""
    return 2 * s.number_of_keys + len(constraint_rows(s)) + 3 * len(point_priors(s))


def _ptr(a, typ):
    return a.ctypes.data_as(C.POINTER(typ)) if a is not None else None


class CProblem:
    """Holds contiguous copies of a problem's arrays and the gba_problem that
    points at them (alive as long as this object)."""

    def __init__(self, s):
        self.keep = []
        p = Problem()
        p.number_of_points = s.number_of_points
        p.number_of_images = s.number_of_images
        p.number_of_cameras = s.number_of_cameras
        p.number_of_keys = s.number_of_keys
        fm = np.ascontiguousarray(s.feature_maps, dtype=np.int64).reshape(-1)
        icm = np.ascontiguousarray(s.image_camera_map, dtype=np.int64).reshape(-1)
        self.keep += [fm, icm]
        p.feature_maps = _ptr(fm, C.c_int64)
        p.image_camera_map = _ptr(icm, C.c_int64)
        p.intrinsic_computations_mask = int(s.intrinsic_mask)
        p.fix_mask = int(s.fix_mask)

        def dbl(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
            self.keep.append(a)
            return _ptr(a, C.c_double)

        p.fix_points = dbl(s.points) if s.fix_mask & FIX_POINTS else None
        p.fix_images = dbl(s.images) if s.fix_mask & FIX_IMAGES else None
        p.fix_cameras = dbl(s.cameras) if s.fix_mask & FIX_CAMERAS else None
        pcs = getattr(s, "point_constraints", None) or []
        ics = getattr(s, "image_constraints", None) or []
        ccs = getattr(s, "camera_constraints", None) or []
        if pcs:
            arr = (PointConstraint * len(pcs))(*[PointConstraint(int(a), int(b), 0) for a, b in pcs])
            self.keep.append(arr)
            p.point_constraints = C.cast(arr, C.POINTER(PointConstraint))
        p.number_of_point_constraints = len(pcs)
        if ics:
            arr = (ImageConstraint * len(ics))(*[ImageConstraint(int(a), int(b), 0) for a, b in ics])
            self.keep.append(arr)
            p.image_constraints = C.cast(arr, C.POINTER(ImageConstraint))
        p.number_of_image_constraints = len(ics)
        if ccs:
            arr = (CameraConstraint * len(ccs))(
                *[CameraConstraint(int(a), int(b), int(c), int(d), 0) for a, b, c, d in ccs])
            self.keep.append(arr)
            p.camera_constraints = C.cast(arr, C.POINTER(CameraConstraint))
        p.number_of_camera_constraints = len(ccs)
        kci = getattr(s, "key_covariance_inverse", None)
        p.key_covariance_inverse = dbl(kci)
        p.constraint_weights = dbl(getattr(s, "constraint_weights", None))
        pri = point_priors(s)
        p.number_of_point_priors = len(pri)
        if pri:
            ids = np.ascontiguousarray(pri, dtype=np.int64)
            self.keep.append(ids)
            p.point_prior_ids = _ptr(ids, C.c_int64)
            p.point_prior_information = dbl(getattr(s, "prior_information", None))
        self.problem = p
        self.x_size = x_size(s)
        self.y_size = y_size(s)
        self.cps = params_per_camera(s.intrinsic_mask)

    @property
    def ref(self):
        return C.byref(self.problem)


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags['C_CONTIGUOUS']
    return a.ctypes.data_as(C.POINTER(C.c_double))
