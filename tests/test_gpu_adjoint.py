"""GPU tests of the discrete adjoint (gp_adjoint): against the CPU adjoint
restatement (tests/adjoint_oracle.py, itself pinned to finite differences
of the oracle) and against central finite differences of the FP64
integration.  Bars: 1e-5 relative against finite differences (1e-6 on the
reference's event-offset case); against the CPU restatement, whose
parameter partials are central differences of the oracle residual, 1e-7 of
the largest gradient entry."""
import numpy as np
import pytest

import adjoint_oracle as AO
from helpers import DT, LY, M, psse_case, synthetic_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _rel(a, b, floor):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


def _close(a, b, tol):
    """max |a - b| <= tol * max |b|"""
    return np.max(np.abs(a - b)) <= tol * np.max(np.abs(b))


@pytest.mark.parametrize("dyr", ["2bus.dyr", "2bus_SEXS.dyr", "2bus_ESDC1A.dyr", "2bus_TGOV1.dyr", "2bus_IEESGO.dyr"])
def test_adjoint_two_bus_against_cpu_adjoint(G, orc, golden_cases, dyr):
    """The reference's adjoint example case (examples/adjoint.jl): 2 buses,
    fault on bus 2 from 0.2 s to 0.3 s, 4.8 s, objective sum dt * w^2; one
    dyr file per exciter and governor model."""
    ps, dp = psse_case(golden_cases, "2bus.raw", dyr)
    PA = LY.ProblemArrays(ps)
    ev = [M.ContingencyEvent(1, 0.02, 0.2, 0.3)]
    ns = LY.jl_round(4.8 / DT)
    idx = AO.differentiated_params(PA)
    J, grad, gz = AO.adjoint(orc, PA, dp.zvec, dp.uvec, dp.pvec, ev, DT, ns, params=idx)
    gbl = G.GpuBatchedLayout(dp, ps, 1)
    try:
        r = gbl.adjoint(4.8, DT, newton_tol=1e-12, scenario_faults=[ev], checkpoint_every=60)
    finally:
        gbl.close()
    assert r["status"][0] == 0
    assert abs(r["J"][0] - J) <= 1e-10 * abs(J)
    assert _close(r["grad_p"][0, idx], grad[idx], 1e-7)
    other = np.setdiff1d(np.arange(PA.n_par), idx)
    assert np.all(r["grad_p"][0, other] == 0.0)
    diff = np.asarray(PA.is_diff, dtype=bool)
    assert _close(r["grad_z0"][0, :diff.size][diff], gz[:diff.size][diff], 1e-7)
    # the event-offset test's parameter: machine H against finite differences
    h = int(PA.tables[0].par_ptr[0] + 6)
    fd = AO.fd_gradient(orc, PA, dp.zvec, dp.uvec, dp.pvec, ev, DT, ns, [h])[0]
    assert abs(r["grad_p"][0, h] - fd) <= 1e-6 * abs(fd)


def test_adjoint_ring39_voltage_penalty_against_cpu_adjoint(G, orc):
    """Machines with SEXS exciters and TGOV1 governors, objective with the
    voltage penalty 10 * max(0, 0.9 - |V|)^2, two fault scenarios."""
    c, w = synthetic_case("ring39", 2)
    ns = 36
    idx = AO.differentiated_params(c.PA)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.adjoint(ns * DT, DT, newton_tol=1e-12, scenario_faults=c.faults, w_volt=10.0, checkpoint_every=7)
    finally:
        gbl.close()
    for m in range(c.M):
        J, grad, gz = AO.adjoint(orc, c.PA, c.dp.zvec, c.dp.uvec, c.dp.pvec, c.faults[m], DT, ns, w_volt=10.0,
                                 params=idx)
        assert abs(r["J"][m] - J) <= 1e-10 * abs(J)
        assert _close(r["grad_p"][m, idx], grad[idx], 1e-7)


def test_adjoint_planar2k_against_fd_and_checkpoints(G):
    """2,000-bus grid (GENROU/GENSAL, SEXS/ESDC1A, IEEEST, TGOV1/IEESGO), two
    fault scenarios, voltage penalty on, 0.5 s: the 20 differentiated
    parameters of largest sensitivity |p dJ/dp| against central differences
    of the GPU's FP64 integration (1e-5), and the same gradient with
    checkpoints every 7 and every 1000 steps."""
    c, w = synthetic_case("planar2k", 2)
    ns = 60
    idx = np.array(AO.differentiated_params(c.PA))
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.adjoint(ns * DT, DT, newton_tol=1e-12, scenario_faults=c.faults, w_volt=10.0, checkpoint_every=7)
        gbl.restore_initial_state()
        r2 = gbl.adjoint(ns * DT, DT, newton_tol=1e-12, scenario_faults=c.faults, w_volt=10.0,
                         checkpoint_every=1000)
    finally:
        gbl.close()
    assert np.array_equal(r["grad_p"], r2["grad_p"]) and np.array_equal(r["J"], r2["J"])
    p0 = c.dp.pvec
    for m in range(c.M):
        sens = np.abs(r["grad_p"][m, idx] * p0[idx])
        pick = idx[np.argsort(sens)[::-1][:20]]
        P = np.tile(p0, (2 * len(pick), 1))
        hs = []
        for q, j in enumerate(pick):
            h = 1e-5 * max(1.0, abs(p0[j]))
            hs.append(h)
            P[2 * q, j] += h
            P[2 * q + 1, j] -= h
        Mf = len(P)
        fd_l = G.GpuBatchedLayout(c.dp, c.ps, Mf, p=P)
        try:
            t = fd_l.integrate(ns * DT, DT, newton_tol=1e-12, scenario_faults=[c.faults[m]] * Mf)["traj"]
        finally:
            fd_l.close()
        Jv = AO.objective_of_traj(c.PA, t, DT, w_volt=10.0)
        fd = np.array([(Jv[2 * q] - Jv[2 * q + 1]) / (2 * hs[q]) for q in range(len(pick))])
        g = r["grad_p"][m, pick]
        err = np.abs(g - fd) / np.abs(fd)
        assert np.max(err) <= 1e-5, (m, list(zip(pick.tolist(), g.tolist(), fd.tolist(), err.tolist())))


def test_adjoint_differentiation_workload_against_fd(G):
    """The differentiation workload as stated: the 2,000-bus grid over 3 s
    (360 steps), checkpoints every 60 steps, objective
    sum dt (sum w^2 + 10 sum max(0, 0.9 - |V|)^2).  Twenty differentiated
    parameters drawn with a fixed seed (not picked by sensitivity) against
    central differences with step h = 1e-6 max(1, |p|) of the FP64
    integration, two fault scenarios.  Bar: |g - fd| <= 1e-5 |fd| + 3 e_fd
    + 1e-6 max |g|, where e_fd = |fd(h) - fd(2h)| estimates the differences'
    own error and the last term the effect of the 1e-12 Newton tolerance
    (the adjoint differentiates the exact backward-Euler equations, the
    differences the iterates that satisfy them to 1e-12: about 1e-7 of the
    largest gradient apart).  At least two of the twenty parameters have
    |fd| above 1e-2 max |g|, so that the relative bar decides for them."""
    c, w = synthetic_case("planar2k_adj", 2)
    ns = 360
    idx = np.array(AO.differentiated_params(c.PA))
    pick = np.sort(np.random.default_rng(2026).choice(idx, size=20, replace=False))
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.adjoint(ns * DT, DT, newton_tol=1e-12, scenario_faults=c.faults, w_volt=10.0, v_min=0.9,
                        checkpoint_every=60)
    finally:
        gbl.close()
    assert np.all(r["status"] == 0)
    p0 = c.dp.pvec
    hs = 1e-6 * np.maximum(1.0, np.abs(p0[pick]))
    for m in range(c.M):
        fds = []
        for scale in (1.0, 2.0):
            P = np.tile(p0, (2 * len(pick), 1))
            for q, j in enumerate(pick):
                P[2 * q, j] += scale * hs[q]
                P[2 * q + 1, j] -= scale * hs[q]
            fd_l = G.GpuBatchedLayout(c.dp, c.ps, len(P), p=P)
            try:
                t = fd_l.integrate(ns * DT, DT, newton_tol=1e-12, scenario_faults=[c.faults[m]] * len(P))["traj"]
            finally:
                fd_l.close()
            Jv = AO.objective_of_traj(c.PA, t, DT, w_volt=10.0)
            del t
            fds.append((Jv[0::2] - Jv[1::2]) / (2 * scale * hs))
        fd, e_fd = fds[0], np.abs(fds[0] - fds[1])
        g = r["grad_p"][m, pick]
        gmax = np.max(np.abs(r["grad_p"][m, idx]))
        ok = np.abs(g - fd) <= 1e-5 * np.abs(fd) + 3.0 * e_fd + 1e-6 * gmax
        bad = ["p[%d]: adjoint %.12e fd %.12e e_fd %.3e rel %.3e" % (j, a, b, e, abs(a - b) / max(abs(b), 1e-300))
               for j, a, b, e, k in zip(pick, g, fd, e_fd, ok) if not k]
        assert not bad, "scenario %d: %s" % (m, "; ".join(bad))
        assert np.sum(np.abs(fd) >= 1e-2 * gmax) >= 2, np.sort(np.abs(fd) / gmax)


def test_adjoint_batch_of_128_equals_single_scenario_runs(G):
    """One call over the 128 scenarios of the differentiation workload: the
    gradients of three of them equal runs of those scenarios alone."""
    c, w = synthetic_case("planar2k_adj", 128)
    kw = dict(newton_tol=1e-10, w_volt=10.0, v_min=0.9, checkpoint_every=60)
    gbl = G.GpuBatchedLayout(c.dp, c.ps, c.M)
    try:
        r = gbl.adjoint(3.0, DT, scenario_faults=c.faults, **kw)
    finally:
        gbl.close()
    assert np.all(r["status"] == 0)
    for m in (0, 57, 127):
        one = G.GpuBatchedLayout(c.dp, c.ps, 1)
        try:
            r1 = one.adjoint(3.0, DT, scenario_faults=[c.faults[m]], **kw)
        finally:
            one.close()
        assert abs(r1["J"][0] - r["J"][m]) <= 1e-12 * abs(r1["J"][0])
        assert np.max(np.abs(r1["grad_p"][0] - r["grad_p"][m])) <= 1e-10 * np.max(np.abs(r1["grad_p"][0]))
