"""CPU tests of the adjoint restatement (tests/adjoint_oracle.py) against
central finite differences of the oracle's integration: the check that the
reference's examples/adjoint.jl and test/test_adjoint_event_offset.jl make
(2-bus case, fault on bus 2 from 0.2 s to 0.3 s with r_f = 0.02, 4.8 s,
objective sum_t dt * sum_gen w^2)."""
import numpy as np
import pytest

import adjoint_oracle as AO
from helpers import DT, LY, M, psse_case


@pytest.fixture(scope="module")
def two_bus(golden_cases, orc):
    ps, dp = psse_case(golden_cases, "2bus.raw", "2bus.dyr")
    PA = LY.ProblemArrays(ps)
    ev = [M.ContingencyEvent(1, 0.02, 0.2, 0.3)]
    ns = LY.jl_round(4.8 / DT)
    J, grad, gz = AO.adjoint(orc, PA, dp.zvec, dp.uvec, dp.pvec, ev, DT, ns)
    return dict(ps=ps, dp=dp, PA=PA, ev=ev, ns=ns, J=J, grad=grad, gz=gz)


def test_adjoint_parameter_gradient_matches_fd(two_bus, orc):
    """Every parameter: dJ/dp by the adjoint against central differences;
    the machine inertia H is the parameter of the event-offset test
    (relative error below 1e-6 there)."""
    c = two_bus
    p = c["dp"].pvec
    idx = list(range(p.size))
    fd = AO.fd_gradient(orc, c["PA"], c["dp"].zvec, c["dp"].uvec, p, c["ev"], DT, c["ns"], idx)
    big = np.abs(fd) > 1e-5
    rel = np.abs(c["grad"][idx] - fd) / np.maximum(np.abs(fd), 1e-12)
    assert big.sum() >= 10
    assert np.max(rel[big]) < 1e-6
    h = c["PA"].tables[0].par_ptr[0] + 6
    assert rel[h] < 1e-6


def test_adjoint_objective_value_matches_trajectory(two_bus, orc):
    c = two_bus
    fa, nf = LY.fault_array([c["ev"]], DT)
    r = orc.integrate(c["PA"], c["dp"].zvec[None, :], c["dp"].uvec[None, :], c["dp"].pvec[None, :], fa, nf, DT,
                      c["ns"], tol=1e-12)
    J = AO.objective_of_traj(c["PA"], r["traj"], DT)[0]
    assert abs(J - c["J"]) <= 1e-12 * abs(J)


def test_adjoint_initial_state_gradient_matches_fd(two_bus, orc):
    """dJ/dz0 on differential states (lambda of examples/adjoint.jl)."""
    c = two_bus
    PA, z0 = c["PA"], c["dp"].zvec
    diff = np.where(np.asarray(PA.is_diff, dtype=bool))[0][:6]
    Z = np.tile(z0, (2 * len(diff), 1))
    hs = []
    for q, i in enumerate(diff):
        h = 1e-6 * max(1.0, abs(z0[i]))
        hs.append(h)
        Z[2 * q, i] += h
        Z[2 * q + 1, i] -= h
    fa, nf = LY.fault_array([c["ev"]] * len(Z), DT)
    r = orc.integrate(PA, Z, np.tile(c["dp"].uvec, (len(Z), 1)), np.tile(c["dp"].pvec, (len(Z), 1)), fa, nf, DT,
                      c["ns"], tol=1e-12, nthreads=8)
    Jv = AO.objective_of_traj(PA, r["traj"], DT)
    fd = np.array([(Jv[2 * q] - Jv[2 * q + 1]) / (2 * hs[q]) for q in range(len(diff))])
    assert np.max(np.abs(c["gz"][diff] - fd)) <= 1e-6 * max(1e-3, np.max(np.abs(fd)))


def test_adjoint_full_model_mix_with_voltage_term(orc):
    """The differentiation workload's objective (speed deviation plus
    10 * max(0, 0.9 - |V|)^2) on a small planar grid with every device type:
    the adjoint's gradient with respect to the differentiated parameters
    (machine H and D, SEXS K, ESDC1A KA, TGOV1 R, IEESGO K1) against central
    differences, through a fault and its clearing."""
    from helpers import synthetic
    w = synthetic._planar("mix", 11, 120, 24, 0.6, 1, 0.5, "random")
    PA = LY.ProblemArrays(w.ps)
    kinds = {r.dtype.kind for r in w.ps.dynamic.devices}
    assert {"genrou", "sexs", "esdc1a", "ieeest", "ieesgo", "tgov1", "zipload"} <= kinds
    ev = w.faults[0]
    ns = LY.jl_round(0.3 / DT)
    fa, nf = LY.fault_array([ev], DT)
    assert 0 < fa[0].on_step < fa[0].off_step <= ns
    idx = AO.differentiated_params(PA)
    kw = dict(w_speed=1.0, w_volt=10.0, v_min=0.9)
    J, grad, _ = AO.adjoint(orc, PA, w.dp.zvec, w.dp.uvec, w.dp.pvec, ev, DT, ns, params=idx, **kw)
    assert J > 0.0
    # the voltage term is active: some bus dips below 0.9 during the fault
    J_speed = AO.adjoint(orc, PA, w.dp.zvec, w.dp.uvec, w.dp.pvec, ev, DT, ns, params=[], **dict(kw, w_volt=0.0))[0]
    assert J > J_speed * (1 + 1e-6)
    fd = AO.fd_gradient(orc, PA, w.dp.zvec, w.dp.uvec, w.dp.pvec, ev, DT, ns, idx, **kw)
    g = grad[idx]
    scale = np.max(np.abs(fd))
    assert scale > 0.0
    assert np.all(np.abs(g - fd) <= 1e-5 * np.abs(fd) + 1e-7 * scale), np.max(np.abs(g - fd) / scale)
