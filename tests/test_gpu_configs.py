"""GPU parity at the full shapes the benchmark numbers are quoted on.

- planar70k, 8 scenarios, the whole 1 s horizon (120 steps): the FP64
  Schur path against the oracle (identical Newton iteration counts, every
  state within 1e-9 relative), and the mixed-precision path against the
  oracle (rotor angle, rotor speed and bus |V| within 1e-6).
- planar2k, 256 scenarios, the whole 2 s horizon (240 steps): the mixed
  path against the FP64 path on every scenario, both against the oracle on
  the first 32 scenarios.

The oracle runs on every host core (OpenMP over scenarios).
"""
import os

import numpy as np
import pytest

from helpers import DT, LY, run_oracle, synthetic_case

pytestmark = pytest.mark.gpu

RTOL = 1e-9      # FP64 path against the oracle, relative per state
TOL = 1e-6       # mixed path: rotor angle, rotor speed, bus |V|
THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _errors(PA, traj, ref):
    g = PA.tables[0]
    d, w = g.diff_ptr + 5, g.diff_ptr + 4
    vr = PA.n_diff + PA.n_alg + 2 * np.arange(PA.n_bus)
    out = [0.0, 0.0, 0.0]
    for m in range(traj.shape[0]):
        vm = np.hypot(traj[m][:, vr], traj[m][:, vr + 1])
        vm_ref = np.hypot(ref[m][:, vr], ref[m][:, vr + 1])
        out[0] = max(out[0], float(np.max(np.abs(traj[m][:, d] - ref[m][:, d]))))
        out[1] = max(out[1], float(np.max(np.abs(traj[m][:, w] - ref[m][:, w]))))
        out[2] = max(out[2], float(np.max(np.abs(vm - vm_ref))))
    return out


def _rel(a, b):
    return max(float(np.max(np.abs(a[m] - b[m]) / np.maximum(1.0, np.abs(b[m])))) for m in range(a.shape[0]))


def _gpu_runs(G, c, nsteps, solvers):
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    out = {}
    try:
        for s in solvers:
            gbl.restore_initial_state()
            out[s] = gbl.integrate(nsteps * DT, DT, scenario_faults=c.faults, solver=s)
    finally:
        gbl.close()
    return out


@pytest.fixture(scope="module")
def planar70k(G, orc):
    c, w = synthetic_case("planar70k", 8)
    runs = _gpu_runs(G, c, 120, (LY.SOLVER_SCHUR_FP64, LY.SOLVER_SCHUR_MIXED))
    o = run_oracle(orc, c, 120, itermax=30, nthreads=THREADS)
    return c, runs, o


def test_planar70k_fp64_full_horizon_matches_oracle(planar70k):
    c, runs, o = planar70k
    g = runs[LY.SOLVER_SCHUR_FP64]
    assert np.all(o["status"] == 0) and np.all(g["status"] == 0)
    assert np.array_equal(g["iters"], o["iters"])
    assert _rel(g["traj"], o["traj"]) <= RTOL


def test_planar70k_mixed_full_horizon_within_1e6_of_oracle(planar70k):
    c, runs, o = planar70k
    g = runs[LY.SOLVER_SCHUR_MIXED]
    assert np.all(g["status"] == 0)
    assert max(_errors(c.PA, g["traj"], o["traj"])) <= TOL


def test_planar2k_256_scenarios_full_horizon(G, orc):
    c, w = synthetic_case("planar2k", 256)
    runs = _gpu_runs(G, c, 240, (LY.SOLVER_SCHUR_FP64, LY.SOLVER_SCHUR_MIXED))
    f64, mx = runs[LY.SOLVER_SCHUR_FP64], runs[LY.SOLVER_SCHUR_MIXED]
    assert np.all(f64["status"] == 0) and np.all(mx["status"] == 0)
    assert max(_errors(c.PA, mx["traj"], f64["traj"])) <= TOL
    sub = type(c)(c.ps, c.dp, c.faults[:32], 32)
    o = run_oracle(orc, sub, 240, itermax=30, nthreads=THREADS)
    assert np.all(o["status"] == 0)
    assert np.array_equal(f64["iters"][:32], o["iters"])
    assert _rel(f64["traj"][:32], o["traj"]) <= RTOL
    assert max(_errors(c.PA, mx["traj"][:32], o["traj"])) <= TOL


@pytest.mark.parametrize("name,M,n_or", [("planar2k_stressed", 64, 8), ("planar70k_charged", 2, 2)])
def test_harder_grids(G, orc, name, M, n_or):
    """The precision form on harder grids: planar2k with four times the loads
    and line charging b ~ U[0, 0.1] pu (2 s), and planar70k with line
    charging b ~ U[0, 0.01] pu (1 s).  The FP64 path against the oracle
    (identical Newton counts, 1e-9), the mixed path against both (1e-6)."""
    c, w = synthetic_case(name, M)
    ns = int(round(w.tf / DT))
    runs = _gpu_runs(G, c, ns, (LY.SOLVER_SCHUR_FP64, LY.SOLVER_SCHUR_MIXED))
    f64, mx = runs[LY.SOLVER_SCHUR_FP64], runs[LY.SOLVER_SCHUR_MIXED]
    assert np.all(f64["status"] == 0) and np.all(mx["status"] == 0)
    assert max(_errors(c.PA, mx["traj"], f64["traj"])) <= TOL
    sub = type(c)(c.ps, c.dp, c.faults[:n_or], n_or)
    o = run_oracle(orc, sub, ns, itermax=30, nthreads=THREADS)
    assert np.all(o["status"] == 0)
    assert np.array_equal(f64["iters"][:n_or], o["iters"])
    assert _rel(f64["traj"][:n_or], o["traj"]) <= RTOL
    assert max(_errors(c.PA, mx["traj"][:n_or], o["traj"])) <= TOL
