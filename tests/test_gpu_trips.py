"""GPU tests of line trips (gp_set_line_trips; TripLineEvent,
src/GradPower.jl:148-167, 500-574, src/dynamics.jl:612-634) in the batched
path, against the oracle's restatement: identical Newton iteration counts
and trajectories within 1e-9 relative on the FP64 path; the mixed path
within 1e-6 of the FP64 path."""
import numpy as np
import pytest

from helpers import DT, LY, M, run_oracle, synthetic_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _case(name, M_):
    c, w = synthetic_case(name, M_)
    br = c.ps.branches
    # per scenario: trip and reclose, permanent trip, none; plus one trip of
    # every scenario later on
    per = []
    for m in range(M_):
        k = (7 * m + 3) % len(br)
        if m % 3 == 0:
            per.append([M.trip_branch_event(br[k], 0.05, 0.15)])
        elif m % 3 == 1:
            per.append([M.trip_branch_event(br[k], 0.125)])
        else:
            per.append([])
    glob = [M.trip_branch_event(br[len(br) // 2], 0.25, 0.3)]
    return c, per, glob


def _gpu(G, c, per, glob, nsteps, solver):
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.integrate(nsteps * DT, DT, scenario_faults=c.faults, solver=solver, trip_events=glob,
                          scenario_trips=per)
    finally:
        gbl.close()
    return r


def _oracle(orc, c, per, glob, nsteps, nthreads=8):
    z, u, p = c.arrays()
    fa, nf = c.fault_array(DT)
    ta, nt = LY.trip_array(per, DT, glob)
    return orc.integrate(c.PA, z, u, p, fa, nf, DT, nsteps, solver=1, itermax=50, nthreads=nthreads, trips=ta,
                         n_trips=nt)


@pytest.mark.parametrize("name,M_", [("ring39", 9), ("planar2k", 6)])
def test_trips_fp64_against_oracle(G, orc, name, M_):
    c, per, glob = _case(name, M_)
    g = _gpu(G, c, per, glob, 40, LY.SOLVER_SCHUR_FP64)
    o = _oracle(orc, c, per, glob, 40)
    # (ring39's third fault scenario hits itermax with or without trips, in
    # the oracle too: compare the converged scenarios)
    assert np.array_equal(g["status"], o["status"])
    ok = o["status"] == 0
    assert ok.sum() >= M_ - 1
    assert np.array_equal(g["iters"][ok], o["iters"][ok])
    assert np.max(np.abs(g["traj"][ok] - o["traj"][ok]) / np.maximum(1.0, np.abs(o["traj"][ok]))) <= 1e-9
    # the trips did something: scenarios with different trips differ
    assert np.max(np.abs(g["traj"][0] - g["traj"][2])) > 1e-6


def test_trips_mixed_against_fp64(G):
    c, per, glob = _case("planar2k", 6)
    g = _gpu(G, c, per, glob, 40, LY.SOLVER_SCHUR_MIXED)
    e = _gpu(G, c, per, glob, 40, LY.SOLVER_SCHUR_FP64)
    assert np.max(np.abs(g["traj"][0] - g["traj"][2])) > 1e-6
    assert np.all(g["status"] == 0) and np.all(e["status"] == 0)
    assert np.max(np.abs(g["traj"] - e["traj"])) <= 1e-6


def test_trips_cleared_and_rejected(G):
    """Trips apply to the calls that pass them; a later call without trips
    runs the intact network; the Woodbury solver and the adjoint refuse
    trips."""
    c, per, glob = _case("ring39", 3)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r0 = gbl.integrate(20 * DT, DT, scenario_faults=c.faults)
        gbl.restore_initial_state()
        gbl.integrate(20 * DT, DT, scenario_faults=c.faults, scenario_trips=per, trip_events=glob)
        with pytest.raises(Exception, match="line trips"):
            gbl.integrate(20 * DT, DT, scenario_faults=c.faults, scenario_trips=per,
                          solver=LY.SOLVER_SHARED_WOODBURY)
        gbl.restore_initial_state()
        r1 = gbl.integrate(20 * DT, DT, scenario_faults=c.faults)
    finally:
        gbl.close()
    assert np.array_equal(r0["traj"], r1["traj"]) and np.array_equal(r0["iters"], r1["iters"])
