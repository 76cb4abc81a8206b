"""ctypes binding of libgba.so (include/gba.h).

There is no CPU fallback: if the library is missing or no CUDA device is
visible, every call raises.  The library is built in-tree by
hs_sfm_gb300/build.py (``python -c "import __graft_entry__ as g; g.build()"``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libgba.so")
_lib = None


class GbaError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = lib().gba_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: {msg} ({status})" if what else f"{msg} ({status})")


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"libgba.so is not built ({LIB_PATH}); run hs_sfm_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    P = C.POINTER(abi.Problem)
    d = C.POINTER(C.c_double)
    O = C.POINTER(abi.Options)
    R = C.POINTER(abi.Report)
    vp = C.c_void_p
    L.gba_status_string.restype = C.c_char_p
    L.gba_status_string.argtypes = [C.c_int]
    L.gba_version.restype = C.c_char_p
    L.gba_kernel_launch_count.restype = C.c_int64
    L.gba_x_size.restype = C.c_int64
    L.gba_x_size.argtypes = [P]
    L.gba_y_size.restype = C.c_int64
    L.gba_y_size.argtypes = [P]
    L.gba_params_per_camera.restype = C.c_int64
    L.gba_params_per_camera.argtypes = [C.c_uint32]
    L.gba_default_options.argtypes = [O]
    L.gba_solve.argtypes = [P, d, O, d, R]
    L.gba_solve_batch.argtypes = [P, C.POINTER(d), C.c_int32, O, C.POINTER(d), R]
    L.gba_solve_batch_into.argtypes = [P, C.POINTER(d), C.c_int32, O, C.POINTER(d), C.POINTER(d), R]
    L.gba_autotune.argtypes = [P, C.POINTER(d), C.POINTER(d), C.c_int32, O, C.POINTER(abi.Tuning)]
    L.gba_plan_create.argtypes = [P, C.POINTER(d), C.c_int32, O, C.POINTER(vp)]
    L.gba_plan_destroy.argtypes = [vp]
    L.gba_plan_number_of_problems.argtypes = [vp]
    L.gba_plan_set_initial_x.argtypes = [vp, C.c_int32, d]
    L.gba_plan_run.argtypes = [vp]
    L.gba_plan_synchronize.argtypes = [vp]
    L.gba_plan_get_x.argtypes = [vp, C.c_int32, d]
    L.gba_plan_get_report.argtypes = [vp, C.c_int32, R]
    L.gba_plan_set_initial_x_all.argtypes = [vp, C.POINTER(d)]
    L.gba_batch_create.argtypes = [P, C.POINTER(d), C.c_int32, O, C.POINTER(vp)]
    L.gba_batch_submit.argtypes = [vp, C.POINTER(d)]
    L.gba_batch_poll.argtypes = [vp, C.POINTER(d), R]
    L.gba_batch_destroy.argtypes = [vp]
    L.gba_plan_get_all.argtypes = [vp, C.POINTER(d), R]
    L.gba_plan_last_run_ms.argtypes = [vp, d]
    L.gba_plan_kernel_stats.argtypes = [vp, C.c_int32, d, C.POINTER(C.c_int32)]
    L.gba_plan_last_run_launches.argtypes = [vp, C.POINTER(C.c_int64)]
    L.gba_vector_function.argtypes = [P, d, d, C.c_int32]
    L.gba_jacobian.argtypes = [P, d, d, d, d, C.c_int32]
    L.gba_cost.argtypes = [P, d, d, O, d]
    L.gba_schur_step.argtypes = [P, d, d, C.c_double, O, d]
    L.gba_plan_query.argtypes = [vp]
    L.gba_plan_device_bytes.argtypes = [vp, C.POINTER(C.c_int64)]
    L.gba_plan_structure.argtypes = [vp, C.POINTER(abi.PlanStructure)]
    SC = C.POINTER(abi.ServerConfig)
    L.gba_default_server_config.argtypes = [SC]
    L.gba_default_server_config.restype = None
    L.gba_server_create.argtypes = [SC, C.POINTER(vp)]
    L.gba_server_destroy.argtypes = [vp]
    L.gba_server_submit.argtypes = [vp, P, d, d, C.POINTER(C.c_int64)]
    L.gba_server_poll.argtypes = [vp, C.c_int64, d, R]
    L.gba_server_wait.argtypes = [vp, C.c_int64, C.c_double, d, R]
    L.gba_server_cancel.argtypes = [vp, C.c_int64]
    L.gba_server_get_stats.argtypes = [vp, C.POINTER(abi.ServerStats)]
    L.gba_estimate_device_bytes.restype = C.c_int64
    L.gba_estimate_device_bytes.argtypes = [P, C.c_int32]
    L.gba_triangulate.argtypes = [C.POINTER(abi.Triangulation), O, d, C.POINTER(C.c_int32)]
    L.gba_triangulate_last_kernel_ms.restype = C.c_double
    L.gba_fma_peak.argtypes = [C.c_int32, C.c_int32, d]
    _lib = L
    return L


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _check(status, what):
    if status != abi.GBA_OK:
        raise GbaError(status, what)


def solve(scene, options=None, x0=None, near_y=None):
    """One problem through gba_solve (host buffers).  Returns (x, report)."""
    L = lib()
    cp = abi.CProblem(scene)
    x = _f64(scene.x0 if x0 is None else x0).copy()
    y = _f64(scene.near_y if near_y is None else near_y)
    opt = options if options is not None else abi.make_options()
    rep = abi.Report()
    st = L.gba_solve(cp.ref, abi.dptr(y), C.byref(opt), abi.dptr(x), C.byref(rep))
    _check(st, "gba_solve")
    return x, rep


def solve_batch(scenes, options=None):
    L = lib()
    cps = [abi.CProblem(s) for s in scenes]
    arr = (abi.Problem * len(cps))(*[c.problem for c in cps])
    ys = [_f64(s.near_y) for s in scenes]
    x0 = [_f64(s.x0) for s in scenes]
    # results in fresh arrays (the library's parallel scatter touches them
    # first); the scenes' x0 are read in place
    xs = [np.empty(c.x_size) for c in cps]
    yp = (C.POINTER(C.c_double) * len(ys))(*[abi.dptr(y) for y in ys])
    x0p = (C.POINTER(C.c_double) * len(x0))(*[abi.dptr(x) for x in x0])
    xp = (C.POINTER(C.c_double) * len(xs))(*[abi.dptr(x) for x in xs])
    reps = (abi.Report * len(scenes))()
    opt = options if options is not None else abi.make_options()
    st = L.gba_solve_batch_into(arr, yp, len(scenes), C.byref(opt), x0p, xp, reps)
    _check(st, "gba_solve_batch_into")
    return xs, list(reps)


def autotune(scenes, options=None):
    """gba_autotune: the work-item sizes (pair_item, image_item, key_item)
    and the Z layout that run the batch fastest, timed on the device;
    returns a dict with the choice, its time per LM iteration and that of
    the defaults."""
    L = lib()
    if not isinstance(scenes, (list, tuple)):
        scenes = [scenes]
    cps = [abi.CProblem(s) for s in scenes]
    arr = (abi.Problem * len(cps))(*[c.problem for c in cps])
    ys = [_f64(s.near_y) for s in scenes]
    x0 = [_f64(s.x0) for s in scenes]
    yp = (C.POINTER(C.c_double) * len(ys))(*[abi.dptr(y) for y in ys])
    xp = (C.POINTER(C.c_double) * len(x0))(*[abi.dptr(x) for x in x0])
    opt = options if options is not None else abi.make_options()
    t = abi.Tuning()
    _check(L.gba_autotune(arr, yp, xp, len(scenes), C.byref(opt), C.byref(t)), "gba_autotune")
    return {"pair_item": t.pair_item, "image_item": t.image_item, "key_item": t.key_item,
            "z_layout": t.z_layout, "ms_per_iteration": t.ms_per_iteration,
            "default_ms_per_iteration": t.default_ms_per_iteration, "candidates": t.candidates}


class Plan:
    """A batch of problems resident on the device (gba_plan_*)."""

    def __init__(self, scenes, options=None):
        L = lib()
        if not isinstance(scenes, (list, tuple)):
            scenes = [scenes]
        self.scenes = list(scenes)
        self._cps = [abi.CProblem(s) for s in self.scenes]
        self._arr = (abi.Problem * len(self._cps))(*[c.problem for c in self._cps])
        self._ys = [_f64(s.near_y) for s in self.scenes]
        yp = (C.POINTER(C.c_double) * len(self._ys))(*[abi.dptr(y) for y in self._ys])
        self.options = options if options is not None else abi.make_options()
        h = C.c_void_p()
        _check(L.gba_plan_create(self._arr, yp, len(self.scenes), C.byref(self.options),
                                 C.byref(h)), "gba_plan_create")
        self.h = h
        self.set_initial_x_all([s.x0 for s in self.scenes])

    def set_initial_x_all(self, x0s):
        """Every problem's x0 in one upload (gba_plan_set_initial_x_all)."""
        xs = [_f64(x) for x in x0s]
        xp = (C.POINTER(C.c_double) * len(xs))(*[abi.dptr(x) for x in xs])
        _check(lib().gba_plan_set_initial_x_all(self.h, xp), "set_initial_x_all")

    def get_all(self):
        """Every problem's (x, report) in one gather (gba_plan_get_all)."""
        xs = [np.zeros(c.x_size) for c in self._cps]
        xp = (C.POINTER(C.c_double) * len(xs))(*[abi.dptr(x) for x in xs])
        reps = (abi.Report * len(xs))()
        _check(lib().gba_plan_get_all(self.h, xp, reps), "get_all")
        return xs, list(reps)

    def set_initial_x(self, q, x0):
        x0 = _f64(x0)
        _check(lib().gba_plan_set_initial_x(self.h, q, abi.dptr(x0)), "set_initial_x")

    def run(self):
        _check(lib().gba_plan_run(self.h), "gba_plan_run")

    def synchronize(self):
        _check(lib().gba_plan_synchronize(self.h), "gba_plan_synchronize")

    def x(self, q=0):
        out = np.zeros(self._cps[q].x_size)
        _check(lib().gba_plan_get_x(self.h, q, abi.dptr(out)), "get_x")
        return out

    def report(self, q=0):
        r = abi.Report()
        _check(lib().gba_plan_get_report(self.h, q, C.byref(r)), "get_report")
        return r

    def last_run_ms(self):
        v = C.c_double()
        _check(lib().gba_plan_last_run_ms(self.h, C.byref(v)), "last_run_ms")
        return v.value

    def stage_ms(self, stage):
        v = C.c_double()
        n = C.c_int32()
        _check(lib().gba_plan_kernel_stats(self.h, stage, C.byref(v), C.byref(n)), "kernel_stats")
        return v.value

    def launches(self):
        v = C.c_int64()
        _check(lib().gba_plan_last_run_launches(self.h, C.byref(v)), "launches")
        return v.value

    def query(self):
        """True when the last run has finished on the device (non-blocking)."""
        st = lib().gba_plan_query(self.h)
        if st == abi.GBA_ERR_BUSY:
            return False
        _check(st, "gba_plan_query")
        return True

    def device_bytes(self):
        v = C.c_int64()
        _check(lib().gba_plan_device_bytes(self.h, C.byref(v)), "device_bytes")
        return v.value

    def structure(self):
        """Sizes of the plan's work lists (keys, key pairs, assembly items, ...)."""
        v = abi.PlanStructure()
        _check(lib().gba_plan_structure(self.h, C.byref(v)), "structure")
        return v.as_dict()

    def close(self):
        if getattr(self, "h", None):
            lib().gba_plan_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_device_bytes(scene, precision=abi.PRECISION_FP64):
    cp = abi.CProblem(scene)
    return int(lib().gba_estimate_device_bytes(cp.ref, precision))


def default_server_config(**solve_options):
    cfg = abi.ServerConfig()
    lib().gba_default_server_config(C.byref(cfg))
    if solve_options:
        cfg.solve = abi.make_options(**solve_options)
    return cfg


class Server:
    """Continuous-batching request loop (gba_server_*).

    submit() copies the request and returns a ticket; poll() / wait() return
    (x, report) once it is solved, or None while it is queued or running."""

    def __init__(self, config=None, **fields):
        self.config = config if config is not None else default_server_config()
        for k, v in fields.items():
            setattr(self.config, k, v)
        h = C.c_void_p()
        _check(lib().gba_server_create(C.byref(self.config), C.byref(h)), "gba_server_create")
        self.h = h
        self._sizes = {}

    def submit(self, scene, x0=None, near_y=None):
        cp = abi.CProblem(scene)
        y = _f64(scene.near_y if near_y is None else near_y)
        x0 = _f64(scene.x0 if x0 is None else x0)
        t = C.c_int64()
        _check(lib().gba_server_submit(self.h, cp.ref, abi.dptr(y), abi.dptr(x0), C.byref(t)),
               "gba_server_submit")
        self._sizes[t.value] = cp.x_size
        return t.value

    def _result(self, st, ticket, out, rep):
        if st == abi.GBA_ERR_BUSY:
            return None
        self._sizes.pop(ticket, None)
        _check(st, "gba_server result")
        return out, rep

    def poll(self, ticket):
        out = np.zeros(self._sizes.get(ticket, 0))
        rep = abi.Report()
        st = lib().gba_server_poll(self.h, ticket, abi.dptr(out), C.byref(rep))
        return self._result(st, ticket, out, rep)

    def wait(self, ticket, timeout_ms=-1.0):
        out = np.zeros(self._sizes.get(ticket, 0))
        rep = abi.Report()
        st = lib().gba_server_wait(self.h, ticket, float(timeout_ms), abi.dptr(out), C.byref(rep))
        return self._result(st, ticket, out, rep)

    def cancel(self, ticket):
        _check(lib().gba_server_cancel(self.h, ticket), "gba_server_cancel")

    def stats(self):
        s = abi.ServerStats()
        _check(lib().gba_server_get_stats(self.h, C.byref(s)), "gba_server_get_stats")
        return s.as_dict()

    def close(self):
        if getattr(self, "h", None):
            lib().gba_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def vector_function(scene, x, precision=abi.PRECISION_FP64):
    cp = abi.CProblem(scene)
    x = _f64(x)
    y = np.zeros(abi.y_size(scene))   # keys, then the constraint rows
    _check(lib().gba_vector_function(cp.ref, abi.dptr(x), abi.dptr(y), precision),
           "gba_vector_function")
    return y


def jacobian(scene, x, precision=abi.PRECISION_FP64, camera=False):
    """Per-key blocks (jp [K,2,3], ji [K,2,6]; with camera=True also the
    free cameras' jc [K,2,cps])."""
    cp = abi.CProblem(scene)
    x = _f64(x)
    K = scene.number_of_keys
    jp = np.zeros((K, 2, 3))
    ji = np.zeros((K, 2, 6))
    jc = np.zeros((K, 2, max(cp.cps, 1))) if camera else None
    _check(lib().gba_jacobian(cp.ref, abi.dptr(x), abi.dptr(jp), abi.dptr(ji),
                              abi.dptr(jc) if camera else None, precision),
           "gba_jacobian")
    return (jp, ji, jc[:, :, :cp.cps]) if camera else (jp, ji)


def cost(scene, x, near_y=None, options=None):
    cp = abi.CProblem(scene)
    x = _f64(x)
    y = _f64(scene.near_y if near_y is None else near_y)
    out = C.c_double()
    opt = options if options is not None else abi.make_options()
    _check(lib().gba_cost(cp.ref, abi.dptr(x), abi.dptr(y), C.byref(opt), C.byref(out)), "gba_cost")
    return out.value


def schur_step(scene, x, mu, near_y=None, options=None):
    cp = abi.CProblem(scene)
    x = _f64(x)
    y = _f64(scene.near_y if near_y is None else near_y)
    dx = np.zeros(cp.x_size)
    opt = options if options is not None else abi.make_options()
    _check(lib().gba_schur_step(cp.ref, abi.dptr(x), abi.dptr(y), mu, C.byref(opt), abi.dptr(dx)),
           "gba_schur_step")
    return dx


def kernel_launch_count():
    return lib().gba_kernel_launch_count()


def triangulate(batch, options=None):
    """Batched multi-view triangulation (gba_triangulate) of a
    synthetic.TriangulationBatch-like object.  Returns (points [n,3],
    per-point status [n])."""
    ct = abi.CTriangulation(batch)
    opt = options if options is not None else abi.make_options()
    pts = np.zeros((ct.n, 3))
    st = np.zeros(ct.n, dtype=np.int32)
    _check(lib().gba_triangulate(ct.ref, C.byref(opt), abi.dptr(pts),
                                 st.ctypes.data_as(C.POINTER(C.c_int32))), "gba_triangulate")
    return pts, st


def fma_peak(precision=abi.PRECISION_MIXED, device=0):
    """FP32 (PRECISION_MIXED) or FP64 FMA throughput of the device, TFLOP/s."""
    out = C.c_double()
    _check(lib().gba_fma_peak(precision, device, C.byref(out)), "gba_fma_peak")
    return out.value
