"""GPU batched power flow (gpu.batched_power_flow): the library's Newton
step on the power-flow problem (every generator a StaticGenerator
stand-in, every load constant power), one scenario per batch member.
Against the host restatement of the reference's polar Newton power flow
(model.runpf, src/pflow.jl, pinned on MATPOWER case 9 in the oracle tests)
run on each scenario's scaled data: |V| and angles within 1e-8."""
import copy

import numpy as np
import pytest

from helpers import M, case9_system, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def G():
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu


def _host_pf(ps, ls, gs):
    ps2 = copy.deepcopy(ps)
    for l in ps2.loads:
        l.pd *= ls
        l.qd *= ls
    slack = [i for i, b in enumerate(ps2.buses) if b.type == M.SLACK]
    for g in ps2.gens:
        if g.bus not in slack:
            g.psch *= gs
    vm, va, P, Q = M.runpf(ps2)
    return vm, va


@pytest.mark.parametrize("name", ["case9", "planar2k"])
def test_batched_power_flow_matches_host(G, golden_known, name):
    if name == "case9":
        ps = case9_system(golden_known)
        M.runpf_inplace(ps)
    else:
        ps = synthetic.planar2k().ps
    scales = np.array([0.9, 1.0, 1.05, 1.1])
    r = G.batched_power_flow(ps, scales)
    assert np.all(r["status"] == 0)
    for m, s in enumerate(scales):
        vm, va = _host_pf(ps, s, s)
        assert np.max(np.abs(r["vm"][m] - vm)) <= 1e-8
        assert np.max(np.abs(r["va"][m] - va)) <= 1e-8
    # the base scenario starts at its own solution: no Newton step
    assert r["iters"][1] == 0 and np.all(r["iters"][[0, 2, 3]] > 0)


def test_batched_power_flow_flat_start_case9(G, golden_known):
    ps = case9_system(golden_known)
    v0 = np.array([b.v0m * np.exp(1j * b.v0a) for b in ps.buses])
    flat = np.where(np.array([b.type for b in ps.buses]) == M.PQ, 1.0 + 0j, np.abs(v0) * np.exp(1j * 0.0))
    r = G.batched_power_flow(ps, [1.0, 1.0], v_start=np.stack([flat, flat]))
    assert np.all(r["status"] == 0) and np.all(r["iters"] >= 3)
    vm, va = _host_pf(ps, 1.0, 1.0)
    assert np.max(np.abs(r["vm"][0] - vm)) <= 1e-8 and np.max(np.abs(r["va"][0] - va)) <= 1e-8


def test_scenario_initial_states_are_equilibria(G, orc):
    """Initial conditions of a load sweep (GPU power flows, host device
    init) equal those of the host power flow + init, and each is an
    equilibrium of its scenario: a run from them stays flat."""
    from helpers import DT, LY
    w = synthetic.planar2k()
    ps = w.ps
    scales = np.array([0.95, 1.05])
    z0, u0, p = G.scenario_initial_states(ps, scales)
    for m, s in enumerate(scales):
        ps2 = copy.deepcopy(ps)
        for l in ps2.loads:
            l.pd *= s
            l.qd *= s
        slack = [i for i, b in enumerate(ps2.buses) if b.type == M.SLACK]
        for g in ps2.gens:
            if g.bus not in slack:
                g.psch *= s
        for rec in ps2.dynamic.devices:
            if rec.dtype.kind == "zipload":
                rec.dtype.pinj *= s
                rec.dtype.qinj *= s
        M.runpf_inplace(ps2)
        dp = M.initialize_dynamics(ps2)
        assert np.max(np.abs(z0[m] - dp.zvec)) <= 1e-8 * max(1.0, np.max(np.abs(dp.zvec)))
        assert np.max(np.abs(p[m] - dp.pvec)) <= 1e-8 * max(1.0, np.max(np.abs(dp.pvec)))
    gbl = G.GpuBatchedLayout(w.dp, ps, 2, z0=z0, p=p, u0=u0)
    try:
        r = gbl.integrate(10 * DT, DT)
    finally:
        gbl.close()
    assert np.all(r["status"] == 0) and np.all(r["iters"] == 0)
    assert not np.allclose(z0[0], z0[1])


def _close(a, b, tol):
    return np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("case", ["ring39", "planar2k", "ieee9_v33.raw/2bus_SEXS.dyr",
                                  "ieee9_v33.raw/ieee9bus_gov.dyr"])
def test_gpu_device_init_matches_host_init(G, golden_cases, case):
    """Device initialisation on the GPU (gp_initialize) against the host
    restatement of initialize_dynamics! (model.initialize_dynamics) on the
    same GPU power flows: states, controls and parameters within 1e-11.
    The cases cover GENROU with IEESGO, TGOV1, SEXS, ESDC1A and IEEEST, and
    PV and slack static generators."""
    from helpers import psse_case
    if "/" in case:
        ps, dp = psse_case(golden_cases, *case.split("/"))
    else:
        w = synthetic.WORKLOADS[case]()
        ps, dp = w.ps, w.dp
    scales = np.array([0.92, 1.0, 1.06])
    zg, ug, pg = G.scenario_initial_states(ps, scales, dp=dp)
    zh, uh, ph = G.scenario_initial_states(ps, scales, on_gpu=False)
    assert _close(zg, zh, 1e-11) and _close(ug, uh, 1e-11) and _close(pg, ph, 1e-11)
    assert not np.allclose(zg[0], zg[2])


def test_gpu_device_init_reports_failure(G):
    """A machine asked for an output it cannot give at its terminal voltage
    leaves a residual above 1e-9: gp_initialize fails with GP_E_NUMERIC and
    says how many machines."""
    from gradpower_gb300 import layout as LY
    w = synthetic.ring39()
    gbl = G.GpuBatchedLayout(w.dp, w.ps, 1)
    try:
        A = gbl.arrays
        nb, ng = A.n_bus, A.tables[LY.GP_GENROU].n
        vm = np.ones((1, nb))
        va = np.zeros((1, nb))
        pq = np.zeros((1, ng, 2))
        pq[0, :, 0] = 0.5
        pq[0, 0, 0] = np.inf
        with pytest.raises(Exception, match="1 machine initialisation"):
            gbl.initialize(vm, va, pq)
    finally:
        gbl.close()
