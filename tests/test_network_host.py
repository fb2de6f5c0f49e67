"""Host-side network helpers against the quantities they must equal:
the realified Ybus against the complex product, a trip event's admittance
terms against the Ybus without the line (`create_trip_line_event`,
src/GradPower.jl:500-543), and the power flow posed as a problem of the
library's Newton step (`power_flow_problem`) against the host power flow:
its residual, evaluated by the oracle, vanishes at the power-flow solution
(but on the rows of a slack bus that carries a load, as in the reference).
"""
import numpy as np
import pytest

from helpers import DT, LY, Case, M, psse_case


@pytest.fixture(scope="module")
def ieee9(golden_cases):
    return psse_case(golden_cases, "ieee9_v33.raw", "ieee9bus_gov.dyr")


def test_realify_ybus_is_the_complex_product(ieee9):
    ps, _ = ieee9
    rng = np.random.default_rng(3)
    V = rng.normal(size=ps.nbus) + 1j * rng.normal(size=ps.nbus)
    current = ps.ybus @ V
    x = np.empty(2 * ps.nbus)
    x[0::2], x[1::2] = V.real, V.imag
    y = M.realify_ybus(ps.ybus) @ x
    assert np.max(np.abs(y[0::2] - current.real)) <= 1e-12 * np.max(np.abs(current))
    assert np.max(np.abs(y[1::2] - current.imag)) <= 1e-12 * np.max(np.abs(current))


def test_trip_event_terms_are_the_lines_share_of_ybus(ieee9):
    ps, _ = ieee9
    assert any(br.tap > 0.0 for br in ps.branches)   # transformers too
    for br in ps.branches:
        ext_f, ext_t = ps.buses[br.fr].i, ps.buses[br.to].i
        ev = M.create_trip_line_event(ps, ext_f, ext_t, 0.1, 0.2)
        assert (ev.from_bus, ev.to_bus, ev.ton, ev.toff) == (br.fr, br.to, 0.1, 0.2)
        first = next(b for b in ps.branches if {b.fr, b.to} == {br.fr, br.to})
        rest = [b for b in ps.branches if b is not first]
        without = M.PowerSystem(ps.baseMVA, ps.buses, ps.gens, ps.loads, rest, ps.shunts, dict(ps.busmap))
        M.build_network(without)
        D = (ps.ybus - without.ybus).toarray()
        f, t = first.fr, first.to
        expect = np.zeros_like(D)
        expect[f, f] += ev.yff
        expect[f, t] += ev.yft
        expect[t, f] += ev.ytf
        expect[t, t] += ev.ytt
        assert np.max(np.abs(D - expect)) <= 1e-12 * np.max(np.abs(ps.ybus.data))
    with pytest.raises(ValueError):
        M.create_trip_line_event(ps, ps.buses[0].i, ps.buses[0].i, 0.1)


@pytest.mark.parametrize("raw,dyr", [("ieee9_v33.raw", "ieee9bus_gov.dyr"), ("2bus.raw", "2bus.dyr"),
                                     ("IEEE39.raw", "IEEE39_gov.dyr")])
def test_power_flow_problem_vanishes_at_the_power_flow_solution(orc, golden_cases, raw, dyr):
    if dyr not in golden_cases["dyr"]:
        pytest.skip("no such dynamic case among the fixtures")
    ps, _ = psse_case(golden_cases, raw, dyr)
    ps2, dp2 = M.power_flow_problem(ps)
    kinds = {rec.dtype.kind for rec in ps2.dynamic.devices}
    assert kinds <= {"zipload", "static_gen"}, kinds
    c = Case(ps2, dp2)
    fa, nf = c.fault_array()
    z = np.ascontiguousarray(dp2.zvec)
    f = orc.residual(c.PA, z, z, dp2.uvec, dp2.pvec, fa, nf, np.zeros(1), DT)
    # zero everywhere but, where the slack bus carries a load, on its rows:
    # runpf! stores slack generation as P_inj - P_load (src/pflow.jl:397-417)
    net = c.PA.n_diff + c.PA.n_alg
    slack = next(k for k, b in enumerate(ps.buses) if b.type == M.SLACK)
    slack_rows = {net + 2 * slack, net + 2 * slack + 1}
    rows = set(np.where(np.abs(f) > 1e-9)[0].tolist())
    assert rows <= slack_rows, sorted(rows)
    if not any(ld.bus == slack for ld in ps.loads):
        assert not rows
    # and it does not vanish away from it
    zp = z.copy()
    zp[net + 2] += 1e-3
    fp = orc.residual(c.PA, zp, zp, dp2.uvec, dp2.pvec, fa, nf, np.zeros(1), DT)
    assert np.max(np.abs(fp)) > 1e-5
