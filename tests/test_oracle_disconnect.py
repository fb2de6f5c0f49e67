"""Device disconnections in the oracle (DisconnectDeviceEvent,
src/GradPower.jl:131-146, 672-698; src/dynamics.jl:612-646): an offline
device is skipped by every kernel (`table.online[k] || continue`,
src/kernels/*.jl), so an offline ZIP load removes exactly its current
injection from its bus rows, and an offline exciter leaves its
backward-Euler rows at z - zold (identity Jacobian rows) with every other
row unchanged.  A disconnection at step k equals the run to step k followed
by the dt = 0 re-solve and the rest of the run with the device offline."""
import copy
import dataclasses

import numpy as np

from helpers import DT, LY, M, synthetic_case


def _offline(PA, t, k):
    """A copy of the problem arrays with device k of table t offline."""
    PA2 = copy.copy(PA)
    PA2._struct = None
    PA2.tables = list(PA.tables)
    on = PA.tables[t].online.copy()
    on[k] = 0
    PA2.tables[t] = dataclasses.replace(PA.tables[t], online=on)
    return PA2


def _perturbed(c, seed=3):
    z, u, p = LY.replicate(c.dp, 1)
    rng = np.random.default_rng(seed)
    return z[0] * (1.0 + 1e-3 * rng.standard_normal(z.shape[1])), z[0], u[0], p[0]


def test_offline_zip_load_removes_its_injection(orc):
    c, w = synthetic_case("ring39", 1)
    zz, z0, u, p = _perturbed(c)
    fa, nf = LY.fault_array([[]], DT)
    off = np.zeros(1, np.uint8)
    f_on = orc.residual(c.PA, zz, z0, u, p, fa, nf, off, DT)
    ZL = c.PA.tables[LY.GP_ZIPLOAD]
    net = c.PA.n_diff + c.PA.n_alg
    for k in (0, ZL.n // 2, ZL.n - 1):
        f_off = orc.residual(_offline(c.PA, LY.GP_ZIPLOAD, k), zz, z0, u, p, fa, nf, off, DT)
        b, pp = int(ZL.bus[k]), int(ZL.par_ptr[k])
        # the load's current, from its parameters (zipload kernel restated)
        pl, ql, al, y0r, y0i = p[pp], p[pp + 1], p[pp + 2], p[pp + 7], p[pp + 8]
        vr, vi = zz[net + 2 * b], zz[net + 2 * b + 1]
        den = max(vr * vr + vi * vi, 0.2)
        ir = vr * al * y0r - vi * al * y0i + (1 - al) * (pl * vr - ql * vi) / den
        ii = vr * al * y0i + vi * al * y0r + (1 - al) * (ql * vr + pl * vi) / den
        d = f_off - f_on
        rows = [net + 2 * b, net + 2 * b + 1]
        assert abs(d[rows[0]] - ir) <= 1e-13 and abs(d[rows[1]] - ii) <= 1e-13
        mask = np.ones(d.size, bool)
        mask[rows] = False
        assert np.all(d[mask] == 0.0)


def test_offline_exciter_rows_hold_their_states(orc):
    c, w = synthetic_case("planar2k", 1)
    zz, z0, u, p = _perturbed(c)
    fa, nf = LY.fault_array([[]], DT)
    off = np.zeros(1, np.uint8)
    f_on = orc.residual(c.PA, zz, z0, u, p, fa, nf, off, DT)
    J_on = orc.jacobian_dense(c.PA, zz, u, p, fa, nf, off, DT)
    for t, nd in ((LY.GP_SEXS, 2), (LY.GP_ESDC1A, 3)):
        T = c.PA.tables[t]
        k = T.n // 3
        PA2 = _offline(c.PA, t, k)
        f_off = orc.residual(PA2, zz, z0, u, p, fa, nf, off, DT)
        J_off = orc.jacobian_dense(PA2, zz, u, p, fa, nf, off, DT)
        rows = list(range(int(T.diff_ptr[k]), int(T.diff_ptr[k]) + nd))
        assert np.array_equal(f_off[rows], zz[rows] - z0[rows])
        assert np.array_equal(J_off[rows], np.eye(J_off.shape[1])[rows])
        mask = np.ones(f_on.size, bool)
        mask[rows] = False
        assert np.array_equal(f_off[mask], f_on[mask])
        assert np.array_equal(J_off[mask], J_on[mask])


def test_disconnect_event_equals_run_then_offline(orc):
    """Disconnect a load and an exciter at step 12 of scenario 0; scenario
    1 runs without events.  Scenario 0's trajectory equals the run to step
    12, the dt = 0 re-solve and 12 more steps of the system with both
    devices statically offline; Schur and monolithic restatements agree."""
    c, w = synthetic_case("ring39", 2)
    z, u, p = LY.replicate(c.dp, 2)
    fa, nf = LY.fault_array([[], []], DT)
    ZL = c.PA.tables[LY.GP_ZIPLOAD]
    SX = c.PA.tables[LY.GP_SEXS]
    kz, kx = 4, 2
    evs = [M.DisconnectDeviceEvent(int(ZL.device_index[kz]), 12 * DT),
           M.DisconnectDeviceEvent(int(SX.device_index[kx]), 12 * DT)]
    da, nd = LY.disconnect_array(c.PA, [evs, []], DT)
    assert nd == 2 and da[0].type == LY.GP_ZIPLOAD and da[0].index == kz and da[1].type == LY.GP_SEXS
    r1 = orc.integrate(c.PA, z, u, p, fa, nf, DT, 24, solver=1, disconnects=da, n_disc=nd)
    r0 = orc.integrate(c.PA, z, u, p, fa, nf, DT, 24, solver=0, disconnects=da, n_disc=nd)
    assert np.all(r1["status"] == 0) and np.all(r0["status"] == 0)
    assert np.max(np.abs(r1["traj"] - r0["traj"])) <= 1e-9
    assert np.array_equal(r1["traj"][0, :13], r1["traj"][1, :13])
    assert r1["iters"][0, 2 * 11 + 1] > 0 and r1["iters"][1, 2 * 11 + 1] == 0
    assert np.max(np.abs(r1["traj"][0, -1] - r1["traj"][1, -1])) > 1e-6
    # the same run in two pieces: the offline system from the state after step 12
    PA2 = _offline(_offline(c.PA, LY.GP_ZIPLOAD, kz), LY.GP_SEXS, kx)
    z12 = r1["traj"][0, 12][None, :].copy()
    fa1, nf1 = LY.fault_array([[]], DT)
    rs = orc.integrate(PA2, z12, u[:1], p[:1], fa1, nf1, 0.0, 1, solver=1)   # the dt = 0 re-solve
    rr = orc.integrate(PA2, rs["z"], u[:1], p[:1], fa1, nf1, DT, 12, solver=1)
    assert np.max(np.abs(rr["traj"][0, 1:] - r1["traj"][0, 13:])) <= 1e-12
    assert np.array_equal(rr["iters"][0, 0::2], r1["iters"][0, 2 * 12::2])
