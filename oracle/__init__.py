"""CPU FP64 oracle of the bundle-adjustment path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs load
this package, as the checker or the timed CPU baseline; the product package
hs_sfm_gb300 never imports it.  See gba_oracle.h for what it restates and
what pins it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from hs_sfm_gb300 import abi

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        P = C.POINTER(abi.Problem)
        d = C.POINTER(C.c_double)
        L.oracle_vector_function.argtypes = [P, d, d]
        L.oracle_jacobian.argtypes = [P, d, d, d, d]
        L.oracle_ffd_jacobian.argtypes = [P, d, C.c_double, C.c_double, d, d, d]
        L.oracle_dense_jacobian.argtypes = [P, d, d]
        L.oracle_normal_equation_dense.argtypes = [P, d, d, d, d]
        L.oracle_cost.argtypes = [P, d, d, C.c_int32, C.c_double, d]
        L.oracle_schur_step.argtypes = [P, d, d, C.c_double, C.c_int32, C.c_int32, C.c_double, d]
        L.oracle_lm_solve.argtypes = [P, d, C.POINTER(abi.Options), C.c_int32, d,
                                      C.POINTER(abi.Report)]
        L.oracle_time_faithful_iteration.argtypes = [P, d, d, C.c_double, C.c_int32, d]
        L.oracle_triangulate.argtypes = [C.POINTER(abi.Triangulation), C.POINTER(abi.Options), d,
                                         C.POINTER(C.c_int32)]
        _lib = L
    return _lib


def _chk(err):
    if err != 0:
        raise RuntimeError(f"oracle error {err}")


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def vector_function(scene, x):
    cp = abi.CProblem(scene)
    x = _f64(x)
    y = np.zeros(cp.y_size)
    _chk(lib().oracle_vector_function(cp.ref, abi.dptr(x), abi.dptr(y)))
    return y


def jacobian(scene, x, ffd=None):
    """Per-key blocks (pb [K,2,3], ib [K,2,6], cb [K,2,c]); ffd=(delta,
    min_delta) selects the forward-finite-difference calculator."""
    cp = abi.CProblem(scene)
    K = scene.number_of_keys
    x = _f64(x)
    pb = np.zeros((K, 2, 3))
    ib = np.zeros((K, 2, 6))
    cb = np.zeros((K, 2, max(cp.cps, 1)))
    if ffd is None:
        _chk(lib().oracle_jacobian(cp.ref, abi.dptr(x), abi.dptr(pb), abi.dptr(ib), abi.dptr(cb)))
    else:
        _chk(lib().oracle_ffd_jacobian(cp.ref, abi.dptr(x), ffd[0], ffd[1], abi.dptr(pb),
                                       abi.dptr(ib), abi.dptr(cb)))
    return pb, ib, cb[:, :, :cp.cps]


def dense_jacobian(scene, x):
    cp = abi.CProblem(scene)
    x = _f64(x)
    J = np.zeros((cp.y_size, cp.x_size))
    _chk(lib().oracle_dense_jacobian(cp.ref, abi.dptr(x), abi.dptr(J)))
    return J


def normal_equation_dense(scene, x, near_y):
    cp = abi.CProblem(scene)
    x, y = _f64(x), _f64(near_y)
    N = np.zeros((cp.x_size, cp.x_size))
    g = np.zeros(cp.x_size)
    _chk(lib().oracle_normal_equation_dense(cp.ref, abi.dptr(x), abi.dptr(y), abi.dptr(N),
                                            abi.dptr(g)))
    return N, g


def cost(scene, x, near_y, loss=abi.LOSS_TRIVIAL, huber_delta=1.0):
    cp = abi.CProblem(scene)
    x, y = _f64(x), _f64(near_y)
    out = C.c_double()
    _chk(lib().oracle_cost(cp.ref, abi.dptr(x), abi.dptr(y), loss, huber_delta, C.byref(out)))
    return out.value


def schur_step(scene, x, near_y, mu, faithful=True, loss=abi.LOSS_TRIVIAL, huber_delta=1.0):
    cp = abi.CProblem(scene)
    x, y = _f64(x), _f64(near_y)
    dx = np.zeros(cp.x_size)
    err = lib().oracle_schur_step(cp.ref, abi.dptr(x), abi.dptr(y), mu, int(faithful), loss,
                                  huber_delta, abi.dptr(dx))
    return err, dx


def lm_solve(scene, near_y=None, x0=None, options=None, faithful=False):
    cp = abi.CProblem(scene)
    x = _f64(scene.x0 if x0 is None else x0).copy()
    y = _f64(scene.near_y if near_y is None else near_y)
    opt = options if options is not None else abi.make_options()
    rep = abi.Report()
    err = lib().oracle_lm_solve(cp.ref, abi.dptr(y), C.byref(opt), int(faithful), abi.dptr(x),
                                C.byref(rep))
    return err, x, rep


def time_faithful_iteration(scene, x, mu, row_stride=1):
    cp = abi.CProblem(scene)
    x, y = _f64(x), _f64(scene.near_y)
    sec = np.zeros(6)
    _chk(lib().oracle_time_faithful_iteration(cp.ref, abi.dptr(y), abi.dptr(x), mu, row_stride,
                                              abi.dptr(sec)))
    return sec


def triangulate(batch, options=None):
    """Points [n,3] and per-point status of a synthetic.TriangulationBatch."""
    ct = abi.CTriangulation(batch)
    opt = options if options is not None else abi.make_options()
    pts = np.zeros((ct.n, 3))
    st = np.zeros(ct.n, dtype=np.int32)
    _chk(lib().oracle_triangulate(ct.ref, C.byref(opt), abi.dptr(pts),
                                  st.ctypes.data_as(C.POINTER(C.c_int32))))
    return pts, st
