"""Python mirror of the reference's GPU entry points, over the C ABI.

    gbl = GpuBatchedLayout(dp, ps, M)                     # ext/...:466
    tvec, trajs = integrate_gpu_schur_cudss(gbl, ps, tf)   # ext/...:3008-3080
    tvec, trajs = integrate_gpu_cudss(gbl, ps, tf)         # ext/...:2924-2996

`trajs[m]` is an (n_sys, n_steps+1) array per scenario, like the reference's
`Vector{Matrix{Float64}}`.  Events come from `ps.dynamic.events` (applied to
every scenario, the reference's semantics); `scenario_faults` adds one event
list per scenario.  There is no CPU fallback: a missing or failing library
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Optional, Sequence

import numpy as np

from . import layout as LY
from . import model as Mdl

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgradpower_gb300.so")
_lib = None


class GradPowerError(RuntimeError):
    pass


def library():
    """Load libgradpower_gb300.so (built by build.py / __graft_entry__.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            raise GradPowerError("libgradpower_gb300.so is not built (%s); run build()" % _LIB_PATH)
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        L.gp_abi_version.restype = C.c_int32
        L.gp_last_error.argtypes = [C.c_char_p, C.c_int32]
        L.gp_last_error.restype = C.c_int32
        L.gp_layout_create.argtypes = [vp, C.c_int32, vp, vp, vp, C.POINTER(C.c_void_p)]
        L.gp_layout_destroy.argtypes = [vp]
        L.gp_layout_stats.argtypes = [vp, vp]
        L.gp_set_state.argtypes = [vp, vp]
        L.gp_get_state.argtypes = [vp, vp]
        L.gp_integrate.argtypes = [vp, vp, C.c_int32, vp, vp, vp, vp]
        L.gp_residual.argtypes = [vp, vp, C.c_double, C.c_int32, vp, vp, vp]
        L.gp_last_timing.argtypes = [vp, vp]
        L.gp_restore_initial_state.argtypes = [vp]
        L.gp_reduced_selftest.argtypes = [vp] * 7
        L.gp_cluster_selftest.argtypes = [vp] * 5 + [C.c_double] + [vp] * 4
        L.gp_residual_static.argtypes = [vp, vp, C.c_double, vp]
        L.gp_set_mixed_policy.argtypes = [vp, C.c_int32, C.c_double, C.c_int32, C.c_int32]
        L.gp_set_profiling.argtypes = [vp, C.c_int32]
        L.gp_set_wait_limit.argtypes = [vp, C.c_int32]
        L.gp_set_line_trips.argtypes = [vp, C.c_int32, vp]
        L.gp_set_device_disconnects.argtypes = [vp, C.c_int32, vp]
        L.gp_initialize.argtypes = [vp] * 7
        L.gp_adjoint.argtypes = [vp, vp, C.c_int32, vp, vp, C.c_int32, vp, vp, vp, vp]
        L.gp_recip_check.argtypes = [C.c_int32, vp, vp]
        for f in ("gp_layout_create", "gp_layout_destroy", "gp_layout_stats", "gp_set_state",
                  "gp_get_state", "gp_integrate", "gp_residual", "gp_last_timing",
                  "gp_restore_initial_state", "gp_reduced_selftest", "gp_cluster_selftest",
                  "gp_residual_static", "gp_set_mixed_policy", "gp_set_profiling", "gp_set_wait_limit",
                  "gp_set_line_trips",
                  "gp_set_device_disconnects", "gp_initialize", "gp_adjoint", "gp_recip_check"):
            getattr(L, f).restype = C.c_int32
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        buf = C.create_string_buffer(1024)
        library().gp_last_error(buf, 1024)
        raise GradPowerError("libgradpower_gb300 error %d: %s" % (rc, buf.value.decode(errors="replace")))


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class GpuBatchedLayout:
    """Device-resident batch of M scenarios (ext/GradPowerCUDAExt/
    GradPowerCUDAExt.jl:303-945).  Owns all device memory; `close()` or
    garbage collection releases it."""

    def __init__(self, dp: Mdl.DynamicProblem, ps: Mdl.PowerSystem, M: int,
                 z0: Optional[np.ndarray] = None, p: Optional[np.ndarray] = None,
                 u0: Optional[np.ndarray] = None):
        self.ps = ps
        self.M = int(M)
        self.arrays = LY.ProblemArrays(ps)
        z, u, pp = LY.replicate(dp, self.M)
        if z0 is not None:
            z = np.ascontiguousarray(z0, dtype=np.float64).reshape(self.M, -1)
        if p is not None:
            pp = np.ascontiguousarray(p, dtype=np.float64).reshape(self.M, -1)
        if u0 is not None:
            u = np.ascontiguousarray(u0, dtype=np.float64).reshape(self.M, -1)
        self.n_sys = self.arrays.n_sys
        self.n_par = self.arrays.n_par
        self._keep = (z, u, pp)
        h = C.c_void_p()
        P = self.arrays.as_ctypes()
        _check(library().gp_layout_create(C.addressof(P), self.M, _p(z), _p(u), _p(pp), C.byref(h)))
        self._h = h
        self._trips_set = False
        self._disconnects_set = False

    def close(self):
        if getattr(self, "_h", None):
            library().gp_layout_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self, vm, va, gen_pq, sg_pq=None):
        """Device initialisation of every scenario on the GPU from solved
        power flows (gp_initialize; initialize_dynamics!,
        src/dynamics.jl:123-250): vm, va [M, n_bus]; gen_pq [M, n GENROU, 2]
        each machine's output; sg_pq [M, n static generators, 2] their
        totals.  The layout's parameter vectors give every parameter (each
        scenario's load powers in the ZIP rows).  The result becomes the
        layout's state and initial state; returns (z0, u0, p) copies."""
        M, nb = self.M, self.arrays.n_bus
        v = np.ascontiguousarray(np.stack([np.asarray(vm, dtype=np.float64).reshape(M, nb),
                                           np.asarray(va, dtype=np.float64).reshape(M, nb)], axis=2))
        g = np.ascontiguousarray(gen_pq, dtype=np.float64).reshape(M, -1, 2)
        sg = None if sg_pq is None else np.ascontiguousarray(sg_pq, dtype=np.float64).reshape(M, -1, 2)
        z0 = np.empty((M, self.n_sys))
        u0 = np.empty((M, max(1, self.arrays.n_ctrl)))
        p = np.empty((M, self.n_par))
        _check(library().gp_initialize(self._h, _p(v), _p(g) if g.size else None,
                                       _p(sg) if sg is not None and sg.size else None, _p(z0), _p(u0), _p(p)))
        return z0, u0[:, :self.arrays.n_ctrl], p

    @property
    def z(self) -> np.ndarray:
        out = np.empty((self.M, self.n_sys))
        _check(library().gp_get_state(self._h, _p(out)))
        return out

    @z.setter
    def z(self, value):
        v = np.ascontiguousarray(value, dtype=np.float64).reshape(self.M, self.n_sys)
        _check(library().gp_set_state(self._h, _p(v)))

    def stats(self) -> dict:
        out = np.zeros(8, dtype=np.int64)
        _check(library().gp_layout_stats(self._h, _p(out)))
        keys = ("n_red", "nnz_S", "nnz_LU", "supernodes", "levels", "factor_flops", "sum_w2", "max_front")
        return dict(zip(keys, (int(v) for v in out)))

    def set_mixed_policy(self, max_age: int = 1, rho_max: float = 0.9, exact_after: int = 8, predict: int = 3):
        """Policy of the mixed-precision solver (see gp_set_mixed_policy in
        include/gradpower_gb300.h); predict: degree of the extrapolated first
        iterate of a step, 0 (none) to 3 (cubic)."""
        _check(library().gp_set_mixed_policy(self._h, int(max_age), float(rho_max), int(exact_after), int(predict)))

    def set_wait_limit(self, polls: int = 1 << 20):
        """Polls after which a dataflow wait gives up (see gp_set_wait_limit
        in include/gradpower_gb300.h); the call then raises GradPowerError
        with GP_E_TIMEOUT and the waiting scenarios get status bit 8."""
        _check(library().gp_set_wait_limit(self._h, int(polls)))

    def set_profiling(self, on: bool = True):
        """Host-driven Newton loop with CUDA events around every phase (for
        timing()); off by default: the loop runs on the device (see
        gp_set_profiling in include/gradpower_gb300.h).  Same results."""
        _check(library().gp_set_profiling(self._h, 1 if on else 0))

    def timing(self) -> dict:
        """Device time of the last integrate call (CUDA events on the
        library's stream); by phase only with set_profiling(True)."""
        out = np.zeros(16)
        _check(library().gp_last_timing(self._h, _p(out)))
        return dict(total_ms=float(out[0]), cluster_ms=float(out[1]), network_ms=float(out[2]),
                    factor_ms=float(out[3]), solve_ms=float(out[4]), update_ms=float(out[7]),
                    newton_iters=float(out[5]), launches=float(out[6]),
                    factor_launches=float(out[8]), linear_solves=float(out[9]),
                    refreshes=float(out[10]), exact_iters=float(out[11]),
                    retries=float(out[12]))

    def restore_initial_state(self):
        _check(library().gp_restore_initial_state(self._h))

    def residual(self, zold, dt, faults=(), fault_on=()):
        """Backward-Euler residual at the current state (parity probe)."""
        fa, nf = LY.fault_array([[] for _ in range(self.M)], dt, faults)
        on = np.ascontiguousarray(np.asarray(fault_on, dtype=np.uint8).reshape(-1)) if nf else np.zeros(1, np.uint8)
        f = np.empty((self.M, self.n_sys))
        zo = np.ascontiguousarray(zold, dtype=np.float64).reshape(self.M, self.n_sys)
        _check(library().gp_residual(self._h, _p(zo), float(dt), nf, C.addressof(fa), _p(on), _p(f)))
        return f

    def integrate(self, tf: float, dt: float = 1.0 / 120.0, newton_tol: float = 1e-10,
                  itermax: int = 30, events: Sequence[Mdl.ContingencyEvent] = (),
                  scenario_faults: Optional[Sequence[Sequence[Mdl.ContingencyEvent]]] = None,
                  want_traj: bool = True, solver: int = LY.SOLVER_SCHUR_FP64,
                  traj_out: Optional[np.ndarray] = None, trip_events: Sequence[Mdl.TripLineEvent] = (),
                  scenario_trips: Optional[Sequence[Sequence[Mdl.TripLineEvent]]] = None,
                  disconnect_events: Sequence[Mdl.DisconnectDeviceEvent] = (),
                  scenario_disconnects: Optional[Sequence[Sequence[Mdl.DisconnectDeviceEvent]]] = None):
        """Integrate every scenario from the current state.  `traj_out`, if
        given, is a C-contiguous float64 array [M, n_steps+1, n_sys] (for
        example a pinned buffer) that receives the trajectories.
        `trip_events` (every scenario, the reference's ps.dynamic.trip_events)
        and `scenario_trips` (per scenario) trip lines (gp_set_line_trips);
        `disconnect_events` (every scenario, ps.dynamic.disconnect_events) and
        `scenario_disconnects` take devices offline
        (gp_set_device_disconnects)."""
        nsteps = LY.jl_round(tf / dt)
        per = scenario_faults if scenario_faults is not None else [[] for _ in range(self.M)]
        fa, nf = LY.fault_array(per, dt, events)
        if trip_events or scenario_trips or self._trips_set:
            ta, nt = LY.trip_array(scenario_trips, dt, trip_events)
            _check(library().gp_set_line_trips(self._h, nt, C.addressof(ta)))
            self._trips_set = nt > 0
        if disconnect_events or scenario_disconnects or self._disconnects_set:
            da, nd = LY.disconnect_array(self.arrays, scenario_disconnects, dt, disconnect_events)
            _check(library().gp_set_device_disconnects(self._h, nd, C.addressof(da)))
            self._disconnects_set = nd > 0
        opt = LY.GpOptions(dt, nsteps, newton_tol, itermax, solver)
        if traj_out is not None:
            if (traj_out.shape != (self.M, nsteps + 1, self.n_sys) or traj_out.dtype != np.float64
                    or not traj_out.flags.c_contiguous):
                raise ValueError("traj_out must be a C-contiguous float64 array of shape %s"
                                 % ((self.M, nsteps + 1, self.n_sys),))
            traj = traj_out
        else:
            traj = np.empty((self.M, nsteps + 1, self.n_sys)) if want_traj else None
        iters = np.zeros((self.M, 2 * max(nsteps, 1)), dtype=np.int32)
        status = np.zeros(self.M, dtype=np.int32)
        _check(library().gp_integrate(self._h, C.byref(opt), nf, C.addressof(fa), _p(traj), _p(iters),
                                      _p(status)))
        tvec = np.arange(nsteps + 1) * dt
        return dict(tvec=tvec, traj=traj, iters=iters[:, :2 * nsteps], status=status)

    def adjoint(self, tf: float, dt: float = 1.0 / 120.0, newton_tol: float = 1e-10, itermax: int = 30,
                events: Sequence[Mdl.ContingencyEvent] = (),
                scenario_faults: Optional[Sequence[Sequence[Mdl.ContingencyEvent]]] = None,
                w_speed: float = 1.0, w_volt: float = 0.0, v_min: float = 0.9, checkpoint_every: int = 60):
        """Objective and its gradients for every scenario, by the discrete
        adjoint of the FP64 Schur integration from the current state
        (gp_adjoint in include/gradpower_gb300.h).  Returns J [M], grad_p
        [M, n_par] (H, D, exciter gain, governor droop; zero elsewhere),
        grad_z0 [M, n_sys] and the forward run's status [M]."""
        nsteps = LY.jl_round(tf / dt)
        per = scenario_faults if scenario_faults is not None else [[] for _ in range(self.M)]
        fa, nf = LY.fault_array(per, dt, events)
        opt = LY.GpOptions(dt, nsteps, newton_tol, itermax, LY.SOLVER_SCHUR_FP64)
        obj = LY.GpObjective(w_speed, w_volt, v_min)
        J = np.zeros(self.M)
        gp_ = np.zeros((self.M, max(self.n_par, 1)))
        gz = np.zeros((self.M, self.n_sys))
        status = np.zeros(self.M, dtype=np.int32)
        _check(library().gp_adjoint(self._h, C.byref(opt), nf, C.addressof(fa), C.byref(obj), int(checkpoint_every),
                                    _p(J), _p(gp_), _p(gz), _p(status)))
        return dict(J=J, grad_p=gp_[:, :self.n_par], grad_z0=gz, status=status)


def scenario_shard(M: int, rank: int, world: int):
    """Contiguous scenario range [lo, hi) of one rank.  Scenarios never
    exchange data during a run, so sharding needs no collective until the
    trajectories are gathered at the end."""
    base, extra = divmod(M, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def integrate_gpu_schur_cudss(gbl: GpuBatchedLayout, ps: Mdl.PowerSystem, tf: float,
                              dt: float = 1.0 / 120.0, newton_tol: float = 1e-10,
                              scenario_faults=None):
    """(tvec, trajs): the reference's GPU Schur integrator
    (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:3008-3080)."""
    r = gbl.integrate(tf, dt, newton_tol, 30, ps.dynamic.events, scenario_faults)
    return r["tvec"], [r["traj"][m].T for m in range(gbl.M)]


def integrate_gpu_cudss(gbl: GpuBatchedLayout, ps: Mdl.PowerSystem, tf: float,
                        dt: float = 1.0 / 120.0, newton_tol: float = 1e-10,
                        scenario_faults=None):
    """(tvec, trajs): the reference's monolithic GPU integrator
    (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2924-2996).  The library runs
    the same exact Newton step with the cluster blocks eliminated first."""
    return integrate_gpu_schur_cudss(gbl, ps, tf, dt, newton_tol, scenario_faults)


def integrate_gpu_shared_multi(gbl: GpuBatchedLayout, ps: Mdl.PowerSystem, tf: float, fault_buses, rfaults,
                               ton: float, toff: float, dt: float = 1.0 / 120.0, newton_tol: float = 1e-10):
    """(tvec, trajs): the reference's shared-factor integrator with a
    per-scenario Woodbury correction
    (ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2640-2708): scenario m faults
    bus fault_buses[m] (0-based here) through rfaults[m] from ton to toff;
    the reduced matrix of scenario 0 at the initial state is factored once
    and shared (GP_SOLVER_SHARED_WOODBURY)."""
    if len(fault_buses) != gbl.M or len(rfaults) != gbl.M:
        raise ValueError("one fault bus and rfault per scenario")
    faults = [[Mdl.ContingencyEvent(int(b), float(r), float(ton), float(toff))]
              for b, r in zip(fault_buses, rfaults)]
    r = gbl.integrate(tf, dt, newton_tol, 30, (), faults, solver=LY.SOLVER_SHARED_WOODBURY)
    return r["tvec"], [r["traj"][m].T for m in range(gbl.M)]


def batched_power_flow(ps: Mdl.PowerSystem, load_scale, gen_scale=None, tol: float = 1e-10,
                       itermax: int = 30, v_start=None):
    """Power flows of len(load_scale) scenarios at once on the GPU: scenario
    m scales every load (P and Q) by load_scale[m] and the scheduled output
    of the non-slack generators by gen_scale[m] (default load_scale[m]).
    The library's Newton step runs on Mdl.power_flow_problem(ps) (the
    reference's power flow, src/pflow.jl, in current-injection form), one
    scenario per batch member; the start is ps's bus voltages (or v_start
    [M, n_bus] complex).  Returns dict(vm, va [M, n_bus], v [M, n_bus]
    complex, iters [M], status [M], p_slack [M] the slack bus's output)."""
    load_scale = np.asarray(load_scale, dtype=np.float64).reshape(-1)
    gen_scale = load_scale if gen_scale is None else np.asarray(gen_scale, dtype=np.float64).reshape(-1)
    M_ = load_scale.size
    ps2, dp = Mdl.power_flow_problem(ps)
    psd = ps2.dynamic
    pvec = np.tile(dp.pvec, (M_, 1))
    for rec in psd.devices:
        d = rec.dtype
        if d.kind == "zipload":
            pvec[:, rec.par_ptr] *= load_scale
            pvec[:, rec.par_ptr + 1] *= load_scale
        elif d.kind == "static_gen" and d.bus_type != Mdl.SLACK:
            pvec[:, rec.par_ptr] *= gen_scale
    z0 = np.tile(dp.zvec, (M_, 1))
    net = psd.diff_dim + psd.alg_dim
    if v_start is not None:
        v = np.asarray(v_start, dtype=np.complex128).reshape(M_, ps2.nbus)
        z0[:, net::2] = v.real
        z0[:, net + 1::2] = v.imag
    gbl = GpuBatchedLayout(dp, ps2, M_, z0=z0, p=pvec)
    try:
        dt = 1.0 / 120.0      # no differential states: dt does not enter
        r = gbl.integrate(dt, dt, newton_tol=tol, itermax=itermax)
    finally:
        gbl.close()
    z = r["traj"][:, 1, :]
    v = z[:, net::2] + 1j * z[:, net + 1::2]
    out = dict(v=v, vm=np.abs(v), va=np.angle(v), iters=r["iters"][:, 0].copy(), status=r["status"])
    for rec in psd.devices:
        d = rec.dtype
        if d.kind == "static_gen" and d.bus_type == Mdl.SLACK:
            out["p_slack"] = z[:, rec.alg_ptr].copy()
    return out


def generator_outputs(ps: Mdl.PowerSystem, vm, va, load_scale, gen_scale):
    """Each generator's output in every scenario after its power flow (the
    write-back of apply_pf_solution / runpf_inplace, vectorised over
    scenarios): PV-bus generators share their bus's reactive injection,
    slack-bus generators its active and reactive injection, the others keep
    their scheduled output (active part scaled by gen_scale).  Returns
    psch, qsch [M, n_gens]."""
    vm = np.asarray(vm, dtype=np.float64)
    va = np.asarray(va, dtype=np.float64)
    M_ = vm.shape[0]
    V = vm * np.exp(1j * va)
    S = V * np.conj((ps.ybus.tocsr() @ V.T).T)
    P, Q = S.real.copy(), S.imag.copy()
    for l in ps.loads:
        P[:, l.bus] -= l.pd * load_scale
        Q[:, l.bus] -= l.qd * load_scale
    ng = np.zeros(ps.nbus, dtype=np.int64)
    for g in ps.gens:
        ng[g.bus] += 1
    psch = np.empty((M_, len(ps.gens)))
    qsch = np.empty((M_, len(ps.gens)))
    for k, g in enumerate(ps.gens):
        bt = ps.buses[g.bus].type
        psch[:, k] = P[:, g.bus] / ng[g.bus] if bt == Mdl.SLACK else g.psch * gen_scale
        qsch[:, k] = Q[:, g.bus] / ng[g.bus] if bt in (Mdl.PV, Mdl.SLACK) else g.qsch
    return psch, qsch


def scenario_initial_states(ps: Mdl.PowerSystem, load_scale, gen_scale=None, tol: float = 1e-10,
                            on_gpu: bool = True, dp: Optional[Mdl.DynamicProblem] = None):
    """Per-scenario initial conditions for a parameter sweep over load
    levels: the power flows of every scenario on the GPU
    (batched_power_flow), then each scenario's device initialisation (the
    reference's initialize_dynamics!, src/dynamics.jl:123-250) on its
    solution: on the GPU (gp_initialize; `dp`, the initialised base case,
    gives the layout its representative state and static parameters,
    computed on the host once if not given), or with on_gpu=False on the
    host per scenario (model.initialize_dynamics).  Returns
    (z0 [M, n_sys], u0 [M, n_ctrl], p [M, n_par]) for GpuBatchedLayout."""
    import copy
    load_scale = np.asarray(load_scale, dtype=np.float64).reshape(-1)
    gen_scale = load_scale if gen_scale is None else np.asarray(gen_scale, dtype=np.float64).reshape(-1)
    r = batched_power_flow(ps, load_scale, gen_scale, tol=tol)
    if np.any(r["status"] != 0):
        raise GradPowerError("power flow of scenario(s) %s did not converge" % np.nonzero(r["status"])[0].tolist())
    if on_gpu:
        M_ = load_scale.size
        base = dp if dp is not None else Mdl.initialize_dynamics(copy.deepcopy(ps))
        psch, qsch = generator_outputs(ps, r["vm"], r["va"], load_scale, gen_scale)
        arrays = LY.ProblemArrays(ps)
        devs = ps.dynamic.devices
        G = arrays.tables[LY.GP_GENROU]
        SG = arrays.tables[LY.GP_STATIC_GEN]
        gen_pq = np.zeros((M_, G.n, 2))
        for k, i in enumerate(G.device_index):
            gen_pq[:, k, 0] = psch[:, devs[i].gen]
            gen_pq[:, k, 1] = qsch[:, devs[i].gen]
        sg_pq = np.zeros((M_, SG.n, 2))
        for k, i in enumerate(SG.device_index):
            for gi in devs[i].dtype.gen_idxs:
                sg_pq[:, k, 0] += psch[:, gi]
                sg_pq[:, k, 1] += qsch[:, gi]
        p = np.tile(base.pvec, (M_, 1))
        ZL = arrays.tables[LY.GP_ZIPLOAD]
        p[:, ZL.par_ptr] *= load_scale[:, None]
        p[:, ZL.par_ptr + 1] *= load_scale[:, None]
        gbl = GpuBatchedLayout(base, ps, M_, p=p)
        try:
            return gbl.initialize(r["vm"], r["va"], gen_pq, sg_pq if SG.n else None)
        finally:
            gbl.close()
    slack = {i for i, b in enumerate(ps.buses) if b.type == Mdl.SLACK}
    zs, us, ps_ = [], [], []
    for m in range(load_scale.size):
        s = copy.deepcopy(ps)
        for l in s.loads:
            l.pd *= load_scale[m]
            l.qd *= load_scale[m]
        for g in s.gens:
            if g.bus not in slack:
                g.psch *= gen_scale[m]
        for rec in s.dynamic.devices:
            if rec.dtype.kind == "zipload":
                rec.dtype.pinj *= load_scale[m]
                rec.dtype.qinj *= load_scale[m]
        Mdl.apply_pf_solution(s, r["vm"][m], r["va"][m])
        dp = Mdl.initialize_dynamics(s)
        zs.append(dp.zvec)
        us.append(dp.uvec)
        ps_.append(dp.pvec)
    return np.array(zs), np.array(us), np.array(ps_)


class BatchedLayout(GpuBatchedLayout):
    """The reference's CPU batch container (src/batched.jl:16-72), same
    constructor `BatchedLayout(dp, ps, M)`; here the batch lives on the GPU
    and `integrate_batched` runs the library's Newton step on it."""


def integrate_batched(bl: GpuBatchedLayout, ps: Mdl.PowerSystem, tf: float,
                      dt: float = 1.0 / 120.0, newton_tol: float = 1e-10,
                      scenario_faults=None):
    """(tvec, trajs): the reference's batched integrator
    (src/batched.jl:417-492): exact Newton, a fresh factorisation every
    iteration, at most 30 iterations per solve."""
    return integrate_gpu_schur_cudss(gbl=bl, ps=ps, tf=tf, dt=dt, newton_tol=newton_tol,
                                     scenario_faults=scenario_faults)
