"""ctypes wrapper of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline may use
this module; the product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.gpo_integrate.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, vp, C.c_double, C.c_int,
                                    C.c_double, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp]
        L.gpo_integrate.restype = C.c_int
        L.gpo_integrate_trips.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, vp, C.c_int, vp, C.c_double, C.c_int,
                                          C.c_double, C.c_int, C.c_int, C.c_int, vp, vp, vp, vp, vp]
        L.gpo_integrate_trips.restype = C.c_int
        L.gpo_integrate_events.argtypes = [vp, C.c_int, vp, vp, vp, C.c_int, vp, C.c_int, vp, C.c_int, vp,
                                           C.c_double, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, vp, vp, vp,
                                           vp, vp]
        L.gpo_integrate_events.restype = C.c_int
        L.gpo_residual.argtypes = [vp, vp, vp, vp, vp, C.c_int, vp, vp, C.c_double, vp]
        L.gpo_residual_trips.argtypes = [vp, vp, vp, vp, vp, C.c_int, vp, vp, C.c_double, vp]
        L.gpo_jacobian_dense_trips.argtypes = [vp, vp, vp, vp, C.c_int, vp, vp, C.c_double, vp]
        L.gpo_residual.restype = C.c_int
        L.gpo_jacobian_dense.argtypes = [vp, vp, vp, vp, C.c_int, vp, vp, C.c_double, vp]
        L.gpo_jacobian_dense.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def integrate(PA, z0, u0, p, faults, n_faults, dt, nsteps, tol=1e-10, itermax=50, solver=0,
              nthreads=1, want_traj=True, trips=None, n_trips=0, disconnects=None, n_disc=0):
    """Run M independent integrate! restatements (one per row of z0).
    Returns dict(traj [M, nsteps+1, n_sys] or None, z [M, n_sys],
    iters [M, 2*nsteps], status [M], stats [M, 6])."""
    M = z0.shape[0]
    n = PA.n_sys
    z0 = np.ascontiguousarray(z0, dtype=np.float64)
    u0 = np.ascontiguousarray(u0, dtype=np.float64)
    p = np.ascontiguousarray(p, dtype=np.float64)
    traj = np.zeros((M, nsteps + 1, n)) if want_traj else None
    zf = np.zeros((M, n))
    iters = np.zeros((M, 2 * nsteps), dtype=np.int32)
    status = np.zeros(M, dtype=np.int32)
    stats = np.zeros((M, 6), dtype=np.int64)
    P = PA.as_ctypes()
    if n_disc:
        lib().gpo_integrate_events(C.addressof(P), M, _p(z0), _p(u0), _p(p), n_faults, C.addressof(faults),
                                   n_trips, C.addressof(trips) if n_trips else None, n_disc,
                                   C.addressof(disconnects), dt, nsteps, tol, itermax, solver, nthreads,
                                   _p(traj), _p(zf), _p(iters), _p(status), _p(stats))
    elif n_trips:
        lib().gpo_integrate_trips(C.addressof(P), M, _p(z0), _p(u0), _p(p), n_faults, C.addressof(faults),
                                  n_trips, C.addressof(trips), dt, nsteps, tol, itermax, solver, nthreads,
                                  _p(traj), _p(zf), _p(iters), _p(status), _p(stats))
    else:
        lib().gpo_integrate(C.addressof(P), M, _p(z0), _p(u0), _p(p), n_faults, C.addressof(faults),
                            dt, nsteps, tol, itermax, solver, nthreads, _p(traj), _p(zf), _p(iters),
                            _p(status), _p(stats))
    return dict(traj=traj, z=zf, iters=iters, status=status, stats=stats)


def residual(PA, z, zold, u0, p, faults, n_faults, fault_on, dt):
    f = np.zeros(PA.n_sys)
    on = np.ascontiguousarray(fault_on, dtype=np.uint8) if n_faults else np.zeros(1, np.uint8)
    P = PA.as_ctypes()
    lib().gpo_residual(C.addressof(P), _p(np.ascontiguousarray(z)), _p(np.ascontiguousarray(zold)),
                       _p(np.ascontiguousarray(u0)), _p(np.ascontiguousarray(p)), n_faults,
                       C.addressof(faults), _p(on), dt, _p(f))
    return f


def jacobian_dense(PA, z, u0, p, faults, n_faults, fault_on, dt):
    n = PA.n_sys
    J = np.zeros((n, n))
    on = np.ascontiguousarray(fault_on, dtype=np.uint8) if n_faults else np.zeros(1, np.uint8)
    P = PA.as_ctypes()
    lib().gpo_jacobian_dense(C.addressof(P), _p(np.ascontiguousarray(z)), _p(np.ascontiguousarray(u0)),
                             _p(np.ascontiguousarray(p)), n_faults, C.addressof(faults), _p(on), dt,
                             _p(J))
    return J


def residual_trips(PA, z, zold, u0, p, trips, n_trips, trip_on, dt):
    """Backward-Euler residual with the flagged line trips applied."""
    f = np.zeros(PA.n_sys)
    on = np.ascontiguousarray(trip_on, dtype=np.uint8) if n_trips else np.zeros(1, np.uint8)
    P = PA.as_ctypes()
    lib().gpo_residual_trips(C.addressof(P), _p(np.ascontiguousarray(z)), _p(np.ascontiguousarray(zold)),
                             _p(np.ascontiguousarray(u0)), _p(np.ascontiguousarray(p)), n_trips,
                             C.addressof(trips), _p(on), dt, _p(f))
    return f


def jacobian_dense_trips(PA, z, u0, p, trips, n_trips, trip_on, dt):
    n = PA.n_sys
    J = np.zeros((n, n))
    on = np.ascontiguousarray(trip_on, dtype=np.uint8) if n_trips else np.zeros(1, np.uint8)
    P = PA.as_ctypes()
    lib().gpo_jacobian_dense_trips(C.addressof(P), _p(np.ascontiguousarray(z)), _p(np.ascontiguousarray(u0)),
                                   _p(np.ascontiguousarray(p)), n_trips, C.addressof(trips), _p(on), dt, _p(J))
    return J
