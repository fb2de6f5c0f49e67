"""Failure detection on the GPU, in forms that fault, trap or hang nothing.

- A dataflow wait that runs out: the per-layout poll limit set to one poll
  makes the waits of the factorisation and solve kernels give up at once.
  The kernels then finish, the call returns GP_E_TIMEOUT with status bit 8
  on the scenarios whose waits gave up, and the next call (default limit)
  on the same layout is exact again.
- A non-finite parameter in one scenario: that scenario stops with status
  bit 2 (non-finite residual) where the oracle stops unconverged; the other
  scenarios are untouched and still match the oracle.
- A singular reduced network matrix in one scenario: tripping the only line
  of a bus without load or machine leaves its rows of S empty.  That
  scenario's FP64 factorisation meets a zero pivot (status bit 4) where the
  oracle's sparse LU fails; the other scenarios still match the oracle.
  (The mixed solver may go on with factors kept from before the trip, which
  are not singular, so it is not part of this check.)

The reference is silent on both (src/batched.jl:459, src/numerics.jl:146-166).
"""
import ctypes as C

import numpy as np
import pytest

from helpers import DT, LY, M, run_oracle, synthetic_case

pytestmark = pytest.mark.gpu

GP_E_TIMEOUT = -5


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _integrate_raw(G, gbl, c, nsteps, solver):
    """gp_integrate through the C ABI: return code and status words."""
    lib = G.library()
    fa, nf = c.fault_array()
    opt = LY.GpOptions(DT, nsteps, 1e-10, 30, solver)
    status = np.zeros(c.M, dtype=np.int32)
    rc = lib.gp_integrate(gbl._h, C.byref(opt), nf, C.addressof(fa), None, None,
                          C.c_void_p(status.ctypes.data))
    return rc, status


@pytest.mark.parametrize("solver", [LY.SOLVER_SCHUR_FP64, LY.SOLVER_SCHUR_MIXED])
def test_wait_limit_runs_out_and_layout_recovers(G, orc, solver):
    c, w = synthetic_case("planar2k", 8)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        gbl.set_wait_limit(1)
        rc, status = _integrate_raw(G, gbl, c, 16, solver)   # past the fault at step 12
        assert rc == GP_E_TIMEOUT
        assert np.any(status & 8)
        buf = C.create_string_buffer(512)
        G.library().gp_last_error(buf, 512)
        assert b"iteration limit" in buf.value
        # default limit again: the next call on the same layout is exact
        gbl.set_wait_limit(1 << 20)
        gbl.restore_initial_state()
        r = gbl.integrate(20 * DT, DT, scenario_faults=c.faults, solver=LY.SOLVER_SCHUR_FP64)
    finally:
        gbl.close()
    o = run_oracle(orc, c, 20, itermax=30, nthreads=8)
    assert np.all(r["status"] == 0)
    assert np.array_equal(r["iters"], o["iters"])
    assert np.max(np.abs(r["traj"] - o["traj"]) / np.maximum(1.0, np.abs(o["traj"]))) <= 1e-9


def test_wait_limit_rejects_zero(G):
    c, w = synthetic_case("two_bus", 1)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, 1)
    try:
        with pytest.raises(G.GradPowerError):
            gbl.set_wait_limit(0)
    finally:
        gbl.close()


@pytest.mark.parametrize("solver", [LY.SOLVER_SCHUR_FP64, LY.SOLVER_SCHUR_MIXED])
def test_nan_parameter_stops_only_its_scenario(G, orc, solver):
    c, w = synthetic_case("planar2k", 4)
    z, u, p = c.arrays()
    p = p.copy()
    H = c.PA.tables[LY.GP_GENROU].par_ptr[0] + 6          # inertia of the first machine
    p[1, H] = np.nan
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M, p=p)
    try:
        r = gbl.integrate(20 * DT, DT, scenario_faults=c.faults, solver=solver)
    finally:
        gbl.close()
    fa, nf = c.fault_array()
    o = orc.integrate(c.PA, z, u, p, fa, nf, DT, 20, itermax=30, nthreads=4)
    # the oracle (as the reference) stops the solve unconverged; the GPU
    # path also says why: a non-finite residual (bit 2)
    assert o["status"][1] != 0 and r["status"][1] & 2
    good = [0, 2, 3]
    assert np.all(o["status"][good] == 0) and np.all(r["status"][good] == 0)
    err = np.max(np.abs(r["traj"][good] - o["traj"][good]) / np.maximum(1.0, np.abs(o["traj"][good])))
    assert err <= (1e-9 if solver == LY.SOLVER_SCHUR_FP64 else 1e-6)


def _isolating_trip(ps):
    """The branch of the first bus with one line and neither load nor
    machine (tripping it isolates the bus)."""
    deg = {}
    for b in ps.branches:
        deg[b.fr] = deg.get(b.fr, 0) + 1
        deg[b.to] = deg.get(b.to, 0) + 1
    busy = {l.bus for l in ps.loads} | {g.bus for g in ps.gens}
    bus = next(b for b in range(ps.nbus) if deg.get(b, 0) == 1 and b not in busy)
    return next(br for br in ps.branches if bus in (br.fr, br.to))


def test_isolated_bus_zero_pivot_stops_only_its_scenario(G, orc):
    c, w = synthetic_case("planar2k", 4)
    per = [[], [M.trip_branch_event(_isolating_trip(c.ps), 0.05)], [], []]
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.integrate(20 * DT, DT, scenario_faults=c.faults, solver=LY.SOLVER_SCHUR_FP64, scenario_trips=per)
    finally:
        gbl.close()
    z, u, p = c.arrays()
    fa, nf = c.fault_array(DT)
    ta, nt = LY.trip_array(per, DT, ())
    o = orc.integrate(c.PA, z, u, p, fa, nf, DT, 20, itermax=30, nthreads=4, trips=ta, n_trips=nt)
    assert o["status"][1] != 0 and r["status"][1] & 4
    good = [0, 2, 3]
    assert np.all(o["status"][good] == 0) and np.all(r["status"][good] == 0)
    assert np.array_equal(r["iters"][good], o["iters"][good])
    err = np.max(np.abs(r["traj"][good] - o["traj"][good]) / np.maximum(1.0, np.abs(o["traj"][good])))
    assert err <= 1e-9
