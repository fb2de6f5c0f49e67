"""Why three ring39 scenarios do not converge (CPU, the oracle only).

In scenarios 2, 12 and 35 of the 39-bus batch (64 seeded faults), one
Newton solve during the fault reaches the reference's iteration limit of 30
in the oracle and on the GPU alike.  The cause is the equations, not the
solver:
- in 2 and 12 the backward-Euler system of that step has no solution near
  the previous state.  A Levenberg-Marquardt minimisation of the residual,
  started from the previous state and from perturbations of it, ends at the
  same residual floor (well above the Newton tolerance) with a zero
  gradient and a singular Jacobian: a fold of the network equations
  (voltage collapse under the fault, through the loads' constant-power
  part).  Given 51 to 100 iterations Newton reaches a distant root in 2,
  and none in 12;
- 35 converges, slowly, with 31 to 50 iterations.
The reference's model has the same loads and the same Newton loop, so it
fails on the same steps.
"""
import numpy as np
import pytest

from helpers import DT, synthetic_case, run_oracle

scipy_opt = pytest.importorskip("scipy.optimize")


@pytest.mark.parametrize("m", [2, 12])
def test_failing_step_has_no_solution(orc, m):
    c, w = synthetic_case("ring39", 64)
    cm = type(c)(c.ps, c.dp, [c.faults[m]], 1)
    full = run_oracle(orc, cm, 30, itermax=30)
    assert full["status"][0] == 1
    q = int(np.argmax(full["iters"][0] >= 30))
    assert q % 2 == 0                       # a step solve, not an event re-solve
    k = q // 2                              # the failing solve is step k + 1
    zprev = full["traj"][0, k]
    fa, nf = cm.fault_array()
    on = np.array([1], np.uint8)            # the fault is on during that step
    fun = lambda x: orc.residual(cm.PA, x, zprev, c.dp.uvec, c.dp.pvec, fa, nf, on, DT)
    jac = lambda x: orc.jacobian_dense(cm.PA, x, c.dp.uvec, c.dp.pvec, fa, nf, on, DT)
    floors = []
    for trial in range(3):
        x0 = zprev if trial == 0 else zprev + 0.05 * np.random.default_rng(trial).normal(size=zprev.size)
        r = scipy_opt.least_squares(fun, x0, jac=jac, method="lm", xtol=1e-15, ftol=1e-15, gtol=1e-15,
                                    max_nfev=5000)
        J = jac(r.x)
        floors.append(np.max(np.abs(r.fun)))
        assert np.max(np.abs(J.T @ r.fun)) < 1e-8                      # a stationary point of |f|^2
        assert np.linalg.svd(J, compute_uv=False)[-1] < 1e-6            # with a singular Jacobian
    assert min(floors) > 1e-4                                            # far above the 1e-10 tolerance
    assert max(floors) - min(floors) < 1e-6 * max(floors) + 1e-9         # the same floor from every start


def test_slow_scenario_converges_with_more_iterations(orc):
    c, w = synthetic_case("ring39", 64)
    cm = type(c)(c.ps, c.dp, [c.faults[35]], 1)
    assert run_oracle(orc, cm, 30, itermax=30)["status"][0] == 1
    assert run_oracle(orc, cm, 30, itermax=50)["status"][0] == 0
