"""GPU tests of the shared-factor Woodbury path (GP_SOLVER_SHARED_WOODBURY,
the reference's integrate_gpu_shared_multi!,
ext/GradPowerCUDAExt/GradPowerCUDAExt.jl:2640-2708): the reduced matrix of
scenario 0 at the initial state is factored once and shared; each
scenario's fault enters as a rank-2 Woodbury correction.

Bars: against the oracle's restatement of the same iteration (solver 3: the
frozen matrix with the fault shunt factored directly, which is what the
Woodbury identity inverts) the Newton iteration counts are identical and
the trajectories agree to 1e-9 relative; against exact Newton both are
converged to the same tolerance (1e-8 relative)."""
import numpy as np
import pytest

from helpers import DT, LY, M, run_oracle, synthetic_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _run(G, c, nsteps, solver, itermax=50):
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.integrate(nsteps * DT, DT, itermax=itermax, scenario_faults=c.faults, solver=solver)
        r["timing"] = gbl.timing()
    finally:
        gbl.close()
    return r


def test_woodbury_planar2k_against_oracle(G, orc):
    c, w = synthetic_case("planar2k", 8)
    g = _run(G, c, 40, LY.SOLVER_SHARED_WOODBURY)
    o = run_oracle(orc, c, 40, solver=3, nthreads=8)
    assert np.all(o["status"] == 0) and np.array_equal(g["status"], o["status"])
    assert np.array_equal(g["iters"], o["iters"])
    assert np.max(np.abs(g["traj"] - o["traj"]) / np.maximum(1.0, np.abs(o["traj"]))) <= 1e-9
    # the chord iteration takes more iterations than exact Newton, to the
    # same root
    e = run_oracle(orc, c, 40, solver=1, nthreads=8)
    assert g["iters"].sum() > e["iters"].sum()
    assert np.max(np.abs(g["traj"] - e["traj"]) / np.maximum(1.0, np.abs(e["traj"]))) <= 1e-8
    assert g["timing"]["factor_launches"] == 2 or g["timing"]["factor_launches"] == 1


def test_woodbury_ring39_reports_what_the_oracle_reports(G, orc):
    """On the 39-bus ring the frozen pre-fault matrix does not carry the
    dt = 0 re-solve at fault onset (the chord iteration stalls): both sides
    report the same scenarios as not converged."""
    c, w = synthetic_case("ring39", 8)
    g = _run(G, c, 30, LY.SOLVER_SHARED_WOODBURY, itermax=30)
    o = run_oracle(orc, c, 30, solver=3, itermax=30, nthreads=8)
    assert np.array_equal(g["status"] != 0, o["status"] != 0)
    # up to the fault both agree step by step
    k = 11
    assert np.array_equal(g["iters"][:, :2 * k], o["iters"][:, :2 * k])
    assert np.max(np.abs(g["traj"][:, :k + 1] - o["traj"][:, :k + 1])) <= 1e-9


def test_woodbury_reference_entry_point(G):
    """integrate_gpu_shared_multi(gbl, ps, tf, fault_buses, rfaults, ton,
    toff) with the reference's argument meaning."""
    c, w = synthetic_case("planar2k", 4)
    buses = [f[0].bus for f in c.faults]
    rf = [f[0].rfault for f in c.faults]
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        tvec, trajs = G.integrate_gpu_shared_multi(gbl, c.ps, 30 * DT, buses, rf, 0.1, 0.2, DT)
        gbl.restore_initial_state()
        faults = [[M.ContingencyEvent(b, r, 0.1, 0.2)] for b, r in zip(buses, rf)]
        r = gbl.integrate(30 * DT, DT, 1e-10, 30, (), faults, solver=LY.SOLVER_SHARED_WOODBURY)
    finally:
        gbl.close()
    assert len(tvec) == 31 and len(trajs) == c.M and trajs[0].shape == (gbl.n_sys, 31)
    for m in range(c.M):
        assert np.array_equal(trajs[m], r["traj"][m].T)


def test_woodbury_rejects_two_fault_buses(G):
    c, w = synthetic_case("planar2k", 2)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        faults = [[M.ContingencyEvent(3, 0.1, 0.1, 0.2), M.ContingencyEvent(5, 0.1, 0.3, 0.4)], []]
        with pytest.raises(Exception, match="more than one fault bus"):
            gbl.integrate(10 * DT, DT, scenario_faults=faults, solver=LY.SOLVER_SHARED_WOODBURY)
    finally:
        gbl.close()


def test_woodbury_planar70k_against_fp64_path(G):
    c, w = synthetic_case("planar70k", 2)
    g = _run(G, c, 30, LY.SOLVER_SHARED_WOODBURY)
    e = _run(G, c, 30, LY.SOLVER_SCHUR_FP64)
    assert np.all(g["status"] == 0) and np.all(e["status"] == 0)
    assert np.max(np.abs(g["traj"] - e["traj"]) / np.maximum(1.0, np.abs(e["traj"]))) <= 1e-8
