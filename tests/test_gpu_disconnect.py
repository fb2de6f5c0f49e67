"""GPU tests of device disconnections (gp_set_device_disconnects;
DisconnectDeviceEvent, src/GradPower.jl:131-146, 672-698,
src/dynamics.jl:612-646) in the batched path, against the oracle's
restatement: identical Newton iteration counts and trajectories within
1e-9 relative on the FP64 path; the mixed path within 1e-6 of the FP64
path.  Loads and exciters (SEXS, ESDC1A) are taken offline; devices whose
algebraic rows would lose their equations are refused."""
import numpy as np
import pytest

from helpers import DT, LY, M, synthetic_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _dev(c, t, k):
    return int(c.PA.tables[t].device_index[k % c.PA.tables[t].n])


def _case(name, M_):
    c, w = synthetic_case(name, M_)
    exc = [t for t in (LY.GP_SEXS, LY.GP_ESDC1A) if c.PA.tables[t].n > 0]
    # per scenario: a load, an exciter, both at different steps, or none;
    # plus one load of every scenario later on
    per = []
    for m in range(M_):
        t = exc[m % len(exc)]
        if m % 4 == 0:
            per.append([M.DisconnectDeviceEvent(_dev(c, LY.GP_ZIPLOAD, 3 * m + 1), 0.05)])
        elif m % 4 == 1:
            per.append([M.DisconnectDeviceEvent(_dev(c, t, 2 * m), 0.125)])
        elif m % 4 == 2:
            per.append([M.DisconnectDeviceEvent(_dev(c, LY.GP_ZIPLOAD, 5 * m), 0.075),
                        M.DisconnectDeviceEvent(_dev(c, t, m), 0.15)])
        else:
            per.append([])
    glob = [M.DisconnectDeviceEvent(_dev(c, LY.GP_ZIPLOAD, 7), 0.25)]
    return c, per, glob


def _gpu(G, c, per, glob, nsteps, solver):
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.integrate(nsteps * DT, DT, scenario_faults=c.faults, solver=solver, disconnect_events=glob,
                          scenario_disconnects=per)
    finally:
        gbl.close()
    return r


def _oracle(orc, c, per, glob, nsteps, nthreads=8):
    z, u, p = c.arrays()
    fa, nf = c.fault_array(DT)
    da, nd = LY.disconnect_array(c.PA, per, DT, glob)
    return orc.integrate(c.PA, z, u, p, fa, nf, DT, nsteps, solver=1, itermax=50, nthreads=nthreads,
                         disconnects=da, n_disc=nd)


@pytest.mark.parametrize("name,M_", [("ring39", 9), ("planar2k", 8)])
def test_disconnects_fp64_against_oracle(G, orc, name, M_):
    c, per, glob = _case(name, M_)
    g = _gpu(G, c, per, glob, 40, LY.SOLVER_SCHUR_FP64)
    o = _oracle(orc, c, per, glob, 40)
    # (ring39's third fault scenario hits itermax in the oracle too: compare
    # the converged scenarios)
    assert np.array_equal(g["status"], o["status"])
    ok = o["status"] == 0
    assert ok.sum() >= M_ - 1
    assert np.array_equal(g["iters"][ok], o["iters"][ok])
    assert np.max(np.abs(g["traj"][ok] - o["traj"][ok]) / np.maximum(1.0, np.abs(o["traj"][ok]))) <= 1e-9
    # the disconnections did something: the load's re-solve iterated (an
    # exciter's needs none: at dt = 0 its rows are z - zold whatever its
    # equations), and the trajectories differ from the run without them
    assert g["iters"][0, 2 * 5 + 1] > 0
    ref = _gpu(G, c, [[] for _ in range(M_)], [], 40, LY.SOLVER_SCHUR_FP64)
    for m in (0, 1, 2):
        assert np.max(np.abs(g["traj"][m, -1] - ref["traj"][m, -1])) > 1e-7


def test_disconnects_mixed_against_fp64(G):
    c, per, glob = _case("planar2k", 8)
    g = _gpu(G, c, per, glob, 40, LY.SOLVER_SCHUR_MIXED)
    e = _gpu(G, c, per, glob, 40, LY.SOLVER_SCHUR_FP64)
    assert np.all(g["status"] == 0) and np.all(e["status"] == 0)
    assert np.max(np.abs(g["traj"] - e["traj"])) <= 1e-6


def test_disconnects_cleared_and_rejected(G):
    """Disconnections apply to the calls that pass them, and every call
    starts with all devices online; a machine or a governor (algebraic rows)
    is refused, and so are the Woodbury solver and the adjoint while
    disconnections are set."""
    c, per, glob = _case("ring39", 3)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r0 = gbl.integrate(20 * DT, DT, scenario_faults=c.faults)
        gbl.restore_initial_state()
        ra = gbl.integrate(20 * DT, DT, scenario_faults=c.faults, scenario_disconnects=per, disconnect_events=glob)
        gbl.restore_initial_state()
        rb = gbl.integrate(20 * DT, DT, scenario_faults=c.faults, scenario_disconnects=per, disconnect_events=glob)
        assert np.array_equal(ra["traj"], rb["traj"]) and np.array_equal(ra["iters"], rb["iters"])
        for t in (LY.GP_GENROU, LY.GP_TGOV1):
            with pytest.raises(Exception, match="algebraic rows"):
                gbl.integrate(20 * DT, DT, scenario_faults=c.faults,
                              disconnect_events=[M.DisconnectDeviceEvent(_dev(c, t, 0), 0.05)])
        with pytest.raises(Exception, match="device disconnections"):
            gbl.integrate(20 * DT, DT, scenario_faults=c.faults, scenario_disconnects=per,
                          solver=LY.SOLVER_SHARED_WOODBURY)
        gbl.restore_initial_state()
        r1 = gbl.integrate(20 * DT, DT, scenario_faults=c.faults)
    finally:
        gbl.close()
    assert np.array_equal(r0["traj"], r1["traj"]) and np.array_equal(r0["iters"], r1["iters"])


def test_events_end_with_the_call(G):
    """After a run with line trips and device disconnections the layout holds
    the intact system again: its residual at the final state equals that of
    a layout that never had the events, set to the same state."""
    c, per, glob = _case("ring39", 3)
    trips = [[M.trip_branch_event(c.ps.branches[2], 0.05)]] * 3
    a = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    b = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        a.integrate(20 * DT, DT, scenario_faults=c.faults, scenario_disconnects=per, disconnect_events=glob,
                    scenario_trips=trips, want_traj=False)
        z = a.z
        b.z = z
        zold = z * (1.0 + 1e-6)
        assert np.array_equal(a.residual(zold, DT), b.residual(zold, DT))
    finally:
        a.close()
        b.close()
