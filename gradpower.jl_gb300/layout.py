"""Flatten a set-up power system into the C-ABI problem descriptor.

`ProblemArrays` holds the 0-based struct-of-arrays tables that
`include/gradpower_gb300.h` declares (the reference's `SimulationLayout`
tables, src/layout.jl:61-179, plus the cluster table of src/clusters.jl:16-57
and the complex Ybus of src/network.jl:29-85); `as_ctypes()` builds the
`gp_problem` struct that points into them.  The arrays must outlive every
call that receives the struct.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass
from typing import Dict, List, Sequence

import numpy as np
import scipy.sparse as sp

from . import model as Mdl

GP_GENROU, GP_IEESGO, GP_TGOV1, GP_SEXS, GP_ESDC1A, GP_IEEEST, GP_ZIPLOAD, GP_STATIC_GEN = range(8)
KIND_TO_TYPE = {"genrou": GP_GENROU, "ieesgo": GP_IEESGO, "tgov1": GP_TGOV1, "sexs": GP_SEXS,
                "esdc1a": GP_ESDC1A, "ieeest": GP_IEEEST, "zipload": GP_ZIPLOAD,
                "static_gen": GP_STATIC_GEN}
NTYPES = 8

SOLVER_SCHUR_FP64 = 0
SOLVER_SCHUR_MIXED = 1
SOLVER_SHARED_WOODBURY = 2

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)


class GpDeviceTable(C.Structure):
    _fields_ = [("n", C.c_int32), ("bus", _i32p), ("diff_ptr", _i32p), ("alg_ptr", _i32p),
                ("ctrl_ptr", _i32p), ("par_ptr", _i32p), ("link0", _i32p), ("link1", _i32p),
                ("online", _u8p)]


class GpProblem(C.Structure):
    _fields_ = [("n_bus", C.c_int32), ("n_diff", C.c_int32), ("n_alg", C.c_int32),
                ("n_ctrl", C.c_int32), ("n_par", C.c_int32),
                ("y_nnz", C.c_int32), ("y_rowptr", _i32p), ("y_colidx", _i32p),
                ("y_re", _f64p), ("y_im", _f64p),
                ("adj_rowptr", _i32p), ("adj_colidx", _i32p),
                ("dev", GpDeviceTable * NTYPES),
                ("is_diff", _u8p),
                ("n_clusters", C.c_int32),
                ("cl_w_start", _i32p), ("cl_w_size", _i32p), ("cl_bus", _i32p),
                ("cl_gen", _i32p), ("cl_sg", _i32p), ("cl_gov_type", _i32p), ("cl_gov", _i32p),
                ("cl_exc_type", _i32p), ("cl_exc", _i32p), ("cl_pss", _i32p)]


class GpFault(C.Structure):
    _fields_ = [("scenario", C.c_int32), ("bus", C.c_int32), ("rfault", C.c_double),
                ("on_step", C.c_int32), ("off_step", C.c_int32)]


class GpLineTrip(C.Structure):
    _fields_ = [("scenario", C.c_int32), ("from_bus", C.c_int32), ("to_bus", C.c_int32),
                ("yff", C.c_double * 2), ("yft", C.c_double * 2), ("ytf", C.c_double * 2),
                ("ytt", C.c_double * 2), ("on_step", C.c_int32), ("off_step", C.c_int32)]


def trip_array(trips_per_scenario, dt: float, global_trips=()):
    """The gp_line_trip array: one entry per (scenario, trip), plus
    scenario = -1 entries for trips of every scenario; steps as the
    reference schedules them (Int(round(t/dt)); no reclose: -1)."""
    rows = [(-1, t) for t in global_trips]
    for m, ts in enumerate(trips_per_scenario or ()):
        rows.extend((m, t) for t in ts)
    arr = (GpLineTrip * max(1, len(rows)))()
    for k, (m, t) in enumerate(rows):
        a = arr[k]
        a.scenario, a.from_bus, a.to_bus = m, t.from_bus, t.to_bus
        for name in ("yff", "yft", "ytf", "ytt"):
            v = complex(getattr(t, name))
            getattr(a, name)[0], getattr(a, name)[1] = v.real, v.imag
        a.on_step = jl_round(t.ton / dt)
        a.off_step = jl_round(t.toff / dt) if math.isfinite(t.toff) else -1
    return arr, len(rows)


class GpDeviceDisconnect(C.Structure):
    _fields_ = [("scenario", C.c_int32), ("type", C.c_int32), ("index", C.c_int32), ("on_step", C.c_int32)]


def disconnect_array(PA: "ProblemArrays", per_scenario, dt: float, global_events=()):
    """The gp_device_disconnect array: one entry per (scenario, event), plus
    scenario = -1 entries for events of every scenario; a device is named by
    its table and row (the device's rank among the devices of its type, as
    _set_device_offline! finds it, src/GradPower.jl:684-697); steps as the
    reference schedules them (Int(round(ton/dt)))."""
    rows = [(-1, e) for e in global_events]
    for m, es in enumerate(per_scenario or ()):
        rows.extend((m, e) for e in es)
    arr = (GpDeviceDisconnect * max(1, len(rows)))()
    for k, (m, e) in enumerate(rows):
        t = next((t for t, T in enumerate(PA.tables) if e.device_idx in set(T.device_index.tolist())), None)
        if t is None:
            raise ValueError("no device %d" % e.device_idx)
        a = arr[k]
        a.scenario, a.type, a.index = m, t, PA.table_pos[e.device_idx]
        a.on_step = jl_round(e.ton / dt)
    return arr, len(rows)


class GpObjective(C.Structure):
    """gp_objective: J = sum_t dt * (w_speed * sum_gen w^2
    + w_volt * sum_bus max(0, v_min - |V|)^2)."""
    _fields_ = [("w_speed", C.c_double), ("w_volt", C.c_double), ("v_min", C.c_double)]


class GpOptions(C.Structure):
    _fields_ = [("dt", C.c_double), ("n_steps", C.c_int32), ("newton_tol", C.c_double),
                ("itermax", C.c_int32), ("solver", C.c_int32)]


def _ptr(a, t):
    return a.ctypes.data_as(t) if a is not None and a.size else C.cast(0, t)


@dataclass
class DeviceTableArrays:
    n: int
    bus: np.ndarray
    diff_ptr: np.ndarray
    alg_ptr: np.ndarray
    ctrl_ptr: np.ndarray
    par_ptr: np.ndarray
    link0: np.ndarray
    link1: np.ndarray
    online: np.ndarray
    device_index: np.ndarray   # index into PowerSystemDynamics.devices


class ProblemArrays:
    """All arrays of one problem descriptor (0-based)."""

    def __init__(self, ps: Mdl.PowerSystem):
        psd = ps.dynamic
        devs = psd.devices
        self.n_bus = ps.nbus
        self.n_diff = psd.diff_dim
        self.n_alg = psd.alg_dim
        self.n_ctrl = psd.ctrl_dim
        self.n_par = psd.par_dim
        self.n_sys = self.n_diff + self.n_alg + 2 * self.n_bus
        Y = sp.csr_matrix(ps.ybus)
        Y.sort_indices()
        self.y_rowptr = Y.indptr.astype(np.int32)
        self.y_colidx = Y.indices.astype(np.int32)
        self.y_re = np.ascontiguousarray(Y.data.real, dtype=np.float64)
        self.y_im = np.ascontiguousarray(Y.data.imag, dtype=np.float64)
        adj = ps.adjacency
        self.adj_rowptr = np.zeros(self.n_bus + 1, dtype=np.int32)
        self.adj_rowptr[1:] = np.cumsum([len(a) for a in adj])
        self.adj_colidx = np.array([j for a in adj for j in a], dtype=np.int32)
        links = Mdl.device_links(ps)
        self.tables: List[DeviceTableArrays] = []
        self.table_pos: Dict[int, int] = {}     # device index -> row in its table
        for t in range(NTYPES):
            idx = [i for i, r in enumerate(devs) if KIND_TO_TYPE[r.dtype.kind] == t]
            for k, i in enumerate(idx):
                self.table_pos[i] = k
            a = lambda vals: np.array(vals, dtype=np.int32)
            l0 = []
            for i in idx:
                d = devs[i].dtype
                if t == GP_STATIC_GEN:
                    l0.append(d.bus_type)
                else:
                    l0.append(links[i][0])
            self.tables.append(DeviceTableArrays(
                len(idx),
                a([devs[i].bus for i in idx]),
                a([devs[i].diff_ptr for i in idx]),
                a([devs[i].alg_ptr for i in idx]),
                a([devs[i].ctrl_ptr for i in idx]),
                a([devs[i].par_ptr for i in idx]),
                a(l0),
                a([links[i][1] for i in idx]),
                np.array([1 if devs[i].online else 0 for i in idx], dtype=np.uint8),
                np.array(idx, dtype=np.int64)))
        self.is_diff = psd.is_diff.astype(np.uint8)
        cl = psd.clusters
        self.n_clusters = len(cl)
        self.cl_w_start = np.array([c.w_start for c in cl], dtype=np.int32)
        self.cl_w_size = np.array([c.w_size for c in cl], dtype=np.int32)
        self.cl_bus = np.array([c.bus for c in cl], dtype=np.int32)
        gen, sg, gvt, gv, ext, ex, pss = [], [], [], [], [], [], []
        for c in cl:
            kind = devs[c.gen].dtype.kind
            gen.append(self.table_pos[c.gen] if kind == "genrou" else -1)
            sg.append(self.table_pos[c.gen] if kind == "static_gen" else -1)
            if c.gov >= 0:
                gvt.append(KIND_TO_TYPE[devs[c.gov].dtype.kind]); gv.append(self.table_pos[c.gov])
            else:
                gvt.append(-1); gv.append(-1)
            if c.exc >= 0:
                ext.append(KIND_TO_TYPE[devs[c.exc].dtype.kind]); ex.append(self.table_pos[c.exc])
            else:
                ext.append(-1); ex.append(-1)
            pss.append(self.table_pos[c.pss] if c.pss >= 0 else -1)
        i32 = lambda v: np.array(v, dtype=np.int32)
        self.cl_gen, self.cl_sg = i32(gen), i32(sg)
        self.cl_gov_type, self.cl_gov = i32(gvt), i32(gv)
        self.cl_exc_type, self.cl_exc = i32(ext), i32(ex)
        self.cl_pss = i32(pss)
        self._struct = None

    def as_ctypes(self) -> GpProblem:
        if self._struct is not None:
            return self._struct
        P = GpProblem()
        P.n_bus, P.n_diff, P.n_alg = self.n_bus, self.n_diff, self.n_alg
        P.n_ctrl, P.n_par = self.n_ctrl, self.n_par
        P.y_nnz = int(self.y_colidx.size)
        P.y_rowptr = _ptr(self.y_rowptr, _i32p)
        P.y_colidx = _ptr(self.y_colidx, _i32p)
        P.y_re = _ptr(self.y_re, _f64p)
        P.y_im = _ptr(self.y_im, _f64p)
        P.adj_rowptr = _ptr(self.adj_rowptr, _i32p)
        P.adj_colidx = _ptr(self.adj_colidx, _i32p)
        for t, T in enumerate(self.tables):
            D = P.dev[t]
            D.n = T.n
            D.bus = _ptr(T.bus, _i32p)
            D.diff_ptr = _ptr(T.diff_ptr, _i32p)
            D.alg_ptr = _ptr(T.alg_ptr, _i32p)
            D.ctrl_ptr = _ptr(T.ctrl_ptr, _i32p)
            D.par_ptr = _ptr(T.par_ptr, _i32p)
            D.link0 = _ptr(T.link0, _i32p)
            D.link1 = _ptr(T.link1, _i32p)
            D.online = _ptr(T.online, _u8p)
        P.is_diff = _ptr(self.is_diff, _u8p)
        P.n_clusters = self.n_clusters
        for name in ("cl_w_start", "cl_w_size", "cl_bus", "cl_gen", "cl_sg", "cl_gov_type",
                     "cl_gov", "cl_exc_type", "cl_exc", "cl_pss"):
            setattr(P, name, _ptr(getattr(self, name), _i32p))
        self._struct = P
        return P


def jl_round(x: float) -> int:
    """Julia's `round` (ties to even), which the reference uses for event
    steps (src/dynamics.jl:530-531); Python's round() has the same rule."""
    return int(round(x))


def fault_array(faults_per_scenario: Sequence[Sequence[Mdl.ContingencyEvent]], dt: float,
                global_events: Sequence[Mdl.ContingencyEvent] = ()):
    """Build the gp_fault array: one entry per (scenario, event), plus
    scenario = -1 entries for events that apply to every scenario."""
    rows = []
    for ev in global_events:
        rows.append((-1, ev.bus, ev.rfault, jl_round(ev.ton / dt), jl_round(ev.toff / dt)))
    for m, evs in enumerate(faults_per_scenario):
        for ev in evs:
            rows.append((m, ev.bus, ev.rfault, jl_round(ev.ton / dt), jl_round(ev.toff / dt)))
    arr = (GpFault * max(1, len(rows)))()
    for k, r in enumerate(rows):
        arr[k].scenario, arr[k].bus, arr[k].rfault, arr[k].on_step, arr[k].off_step = r
    return arr, len(rows)


def replicate(dp: Mdl.DynamicProblem, M: int):
    """Scenario-major copies of z0, u0, p (BatchedLayout, src/batched.jl:61-72)."""
    z = np.ascontiguousarray(np.tile(dp.zvec, (M, 1)))
    u = np.ascontiguousarray(np.tile(dp.uvec, (M, 1)))
    p = np.ascontiguousarray(np.tile(dp.pvec, (M, 1)))
    return z, u, p
