"""Line trips in the oracle (TripLineEvent, src/GradPower.jl:148-167,
500-574; src/dynamics.jl:612-634): with the trip applied, the residual
and the Jacobian equal those of the same system built without that line."""
import copy

import numpy as np

from helpers import DT, LY, M, synthetic_case


def _without_branch(ps, k):
    ps2 = copy.copy(ps)
    ps2.branches = [b for i, b in enumerate(ps.branches) if i != k]
    M.build_network(ps2)
    return ps2


def test_trip_residual_and_jacobian_equal_the_system_without_the_line(orc):
    c, w = synthetic_case("ring39", 1)
    ps = c.ps
    z, u, p = LY.replicate(c.dp, 1)
    rng = np.random.default_rng(3)
    zz = z[0] * (1.0 + 1e-3 * rng.standard_normal(z.shape[1]))
    for k in (0, 5, len(ps.branches) - 1):
        ev = M.trip_branch_event(ps.branches[k], 0.1)
        ta, nt = LY.trip_array([[ev]], DT)
        PA2 = LY.ProblemArrays(_without_branch(ps, k))
        fa, nf = LY.fault_array([[]], DT)
        f_trip = orc.residual_trips(c.PA, zz, z[0], u[0], p[0], ta, nt, [1], DT)
        f_ref = orc.residual(PA2, zz, z[0], u[0], p[0], fa, nf, np.zeros(1, np.uint8), DT)
        assert np.max(np.abs(f_trip - f_ref)) <= 1e-12 * max(1.0, np.max(np.abs(f_ref)))
        f_off = orc.residual_trips(c.PA, zz, z[0], u[0], p[0], ta, nt, [0], DT)
        f0 = orc.residual(c.PA, zz, z[0], u[0], p[0], fa, nf, np.zeros(1, np.uint8), DT)
        assert np.array_equal(f_off, f0)
        J_trip = orc.jacobian_dense_trips(c.PA, zz, u[0], p[0], ta, nt, [1], DT)
        J_ref = orc.jacobian_dense(PA2, zz, u[0], p[0], fa, nf, np.zeros(1, np.uint8), DT)
        assert np.max(np.abs(J_trip - J_ref)) <= 1e-12 * np.max(np.abs(J_ref))


def test_trip_and_reclose_integrate(orc):
    """A trip at 0.1 s reclosed at 0.2 s: the state after the reclose
    returns toward the pre-trip equilibrium; a permanent trip does not; the
    Schur and monolithic restatements agree."""
    c, w = synthetic_case("ring39", 2)
    z, u, p = LY.replicate(c.dp, 2)
    fa, nf = LY.fault_array([[], []], DT)
    evs = [M.trip_branch_event(c.ps.branches[3], 0.1, 0.2), M.trip_branch_event(c.ps.branches[3], 0.1)]
    ta, nt = LY.trip_array([[evs[0]], [evs[1]]], DT)
    r1 = orc.integrate(c.PA, z, u, p, fa, nf, DT, 60, solver=1, trips=ta, n_trips=nt)
    r0 = orc.integrate(c.PA, z, u, p, fa, nf, DT, 60, solver=0, trips=ta, n_trips=nt)
    assert np.all(r1["status"] == 0) and np.all(r0["status"] == 0)
    assert np.max(np.abs(r1["traj"] - r0["traj"])) <= 1e-9
    # both scenarios identical up to the reclose; the trip changed the state
    assert np.array_equal(r1["traj"][0, :25], r1["traj"][1, :25])
    assert np.max(np.abs(r1["traj"][0, 13] - r1["traj"][0, 12])) > 1e-6
    assert r1["iters"][0, 2 * 11 + 1] > 0 and r1["iters"][0, 2 * 23 + 1] > 0 and r1["iters"][1, 2 * 23 + 1] == 0
    d_reclosed = np.max(np.abs(r1["traj"][0, -1] - z[0]))
    d_tripped = np.max(np.abs(r1["traj"][1, -1] - z[0]))
    assert d_reclosed < d_tripped
