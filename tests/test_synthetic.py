"""The seeded synthetic grids stand in for the benchmark's stated
configurations: their sizes, model mix and parameter distributions are the
stated ones (the deviations each workload records in its notes aside)."""
import collections

import numpy as np
import pytest

from helpers import synthetic


def _kinds(w):
    return collections.Counter(rec.dtype.kind for rec in w.ps.dynamic.devices)


def _of(w, kind):
    return [rec.dtype for rec in w.ps.dynamic.devices if rec.dtype.kind == kind]


def _salient(g):
    # a GENSAL is a GENROU whose q-axis transient terms are the d-axis ones
    return g.x_qp == g.x_dp and g.T_q0p == g.T_d0p


def _check_machines(gens, H_range, spread):
    base = dict(x_d=1.8, x_q=1.7, x_dp=0.3, x_qp=0.55, xl=0.2, T_d0p=6.0, T_q0p=0.5, T_d0dp=0.03,
                T_q0dp=0.05)
    H = np.array([g.H for g in gens])
    assert H.min() >= H_range[0] and H.max() <= H_range[1]
    assert all(g.D == 0.0 for g in gens)
    for name, v in base.items():
        x = np.array([getattr(g, name) for g in gens if not (_salient(g) and name in ("x_qp", "T_q0p"))])
        assert x.min() >= v * (1 - spread) - 1e-12 and x.max() <= v * (1 + spread) + 1e-12, name


def _check_controls(w):
    for e in _of(w, "sexs"):
        assert (e.TA_TB, e.TB, e.K, e.TE, e.EMIN, e.EMAX) == (0.1, 10.0, 100.0, 0.05, -5.0, 5.0)
    for e in _of(w, "esdc1a"):
        assert (e.Ka, e.Ta, e.Ke, e.Te, e.Kf, e.Tf) == (400.0, 0.02, 1.0, 0.8, 0.03, 1.0)
    for g in _of(w, "tgov1"):
        assert (g.R, g.T1, g.T2, g.T3) == (0.05, 0.5, 1.0, 2.0)
    for g in _of(w, "ieesgo"):
        T = np.array([g.T1, g.T2, g.T3, g.T4, g.T5, g.T6])
        assert T.min() >= 0.05 and T.max() <= 0.5
        assert (g.K1, g.K2, g.K3, g.pmax, g.pmin) == (20.0, 0.5, 0.5, 1.2, 0.0)


def test_ring39_configuration():
    """39-bus ring plus 7 chords (46 branches), 10 GENROU each with SEXS and
    TGOV1, 19 ZIP loads, 64 fault scenarios over 1 s at dt = 1/120."""
    w = synthetic.ring39()
    assert w.ps.nbus == 39 and len(w.ps.branches) == 46
    assert _kinds(w) == {"genrou": 10, "sexs": 10, "tgov1": 10, "zipload": 19}
    assert w.n_scenarios == 64 and len(w.faults) == 64 and w.tf == 1.0 and w.dt == 1.0 / 120.0
    _check_machines(_of(w, "genrou"), (3.0, 10.0), 0.2)
    _check_controls(w)
    br = w.ps.branches
    assert min(b.r for b in br) >= 0.001 and max(b.r for b in br) <= 0.01
    assert min(b.x for b in br) >= 0.01 and max(b.x for b in br) <= 0.1
    # a different seeded fault bus per scenario, cleared after 0.1 s
    fb = [f[0].bus for f in w.faults]
    assert len(set(fb)) > 1
    assert all(abs(f[0].toff - f[0].ton - 0.1) < 1e-12 for f in w.faults)


@pytest.mark.parametrize("name,n_bus,n_gen,load_frac,scen,tf", [
    ("planar2k", 2000, 400, 0.6, 256, 2.0),
    ("planar70k", 70000, 5000, 0.55, 8, 1.0),
])
def test_planar_configuration(name, n_bus, n_gen, load_frac, scen, tf):
    """Random planar grid of mean degree 2.7; machines 60% GENROU, 40%
    GENSAL; SEXS or ESDC1A half each, IEEEST on a quarter, TGOV1 or IEESGO
    half each; ZIP loads on the stated share of buses."""
    w = synthetic.WORKLOADS[name]()
    ps = w.ps
    assert ps.nbus == n_bus
    assert abs(2 * len(ps.branches) / n_bus - 2.7) < 0.01
    k = _kinds(w)
    assert k["genrou"] == n_gen
    assert k["sexs"] + k["esdc1a"] == n_gen and k["tgov1"] + k["ieesgo"] == n_gen
    assert k["zipload"] == int(round(load_frac * n_bus))
    gens = _of(w, "genrou")
    # binomial shares: within four standard deviations of the stated ones
    tol = lambda p: 4 * np.sqrt(p * (1 - p) / n_gen)   # noqa: E731
    assert abs(np.mean([_salient(g) for g in gens]) - 0.4) < tol(0.4)
    assert abs(k["sexs"] / n_gen - 0.5) < tol(0.5)
    assert abs(k["tgov1"] / n_gen - 0.5) < tol(0.5)
    assert abs(k["ieeest"] / n_gen - 0.25) < tol(0.25)
    _check_machines(gens, (3.0, 10.0), 0.2)
    _check_controls(w)
    assert w.n_scenarios == scen and len(w.faults) == scen and w.tf == tf and w.dt == 1.0 / 120.0


def test_two_bus_configuration():
    """Slack bus with one GENROU (H in [3, 6] s, the stated machine constants
    exactly) and an IEESGO governor; a 0.8 + j0.3 pu load on bus 2 (its Q
    stored negated, as the reference's case import stores it); one line of
    r = 0.01, x = 0.1 pu; a 0.2 pu fault on bus 2 from 0.2 s to 0.3 s; 10 s
    at dt = 1/120."""
    w = synthetic.two_bus()
    ps = w.ps
    assert ps.nbus == 2 and ps.buses[0].type == 3
    assert [(b.fr, b.to, b.r, b.x, b.sh) for b in ps.branches] == [(0, 1, 0.01, 0.1, 0.0)]
    assert [(ld.bus, ld.pd, ld.qd) for ld in ps.loads] == [(1, 0.8, -0.3)]
    assert _kinds(w) == {"genrou": 1, "ieesgo": 1, "zipload": 1}
    g = _of(w, "genrou")[0]
    assert 3.0 <= g.H <= 6.0 and g.D == 0.0
    assert (g.x_d, g.x_q, g.x_dp, g.x_qp, g.x_ddp, g.xl) == (1.8, 1.7, 0.3, 0.55, 0.25, 0.2)
    assert (g.T_d0p, g.T_q0p, g.T_d0dp, g.T_q0dp, g.S1, g.S2) == (6.0, 0.5, 0.03, 0.05, 0.09, 0.38)
    _check_controls(w)
    (f,), = w.faults
    assert (f.bus, f.rfault, f.ton, f.toff) == (1, 0.2, 0.2, 0.3)
    assert w.n_scenarios == 1 and w.tf == 10.0 and w.dt == 1.0 / 120.0


@pytest.mark.parametrize("name", ["two_bus", "ring39", "planar2k", "planar2k_adj", "planar2k_stressed",
                                  "planar70k", "planar70k_charged"])
def test_workloads_start_at_an_equilibrium(orc, name):
    """Every workload's initial state is a steady state of its pre-fault
    system: the oracle's backward-Euler residual vanishes there, the
    check the reference makes of initialize_dynamics! (src/dynamics.jl:58,
    test/test_integrate.jl:27-47)."""
    from helpers import DT, Case
    w = synthetic.WORKLOADS[name]()
    c = Case(w.ps, w.dp)
    fa, nf = c.fault_array()
    f = orc.residual(c.PA, w.dp.zvec, w.dp.zvec, w.dp.uvec, w.dp.pvec, fa, nf, np.zeros(1), DT)
    assert np.max(np.abs(f)) < 1e-9
