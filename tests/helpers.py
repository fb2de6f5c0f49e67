"""Case builders shared by the CPU and GPU tests."""
import numpy as np

from conftest import load_package

gp = load_package()
from gradpower_gb300 import layout as LY, model as M, psse, synthetic  # noqa: E402

DT = 1.0 / 120.0


class Case:
    def __init__(self, ps, dp, faults_per_scenario=None, M_=1, events=()):
        self.ps = ps
        self.dp = dp
        self.PA = LY.ProblemArrays(ps)
        self.M = M_
        self.faults = faults_per_scenario if faults_per_scenario is not None else [[] for _ in range(M_)]
        self.events = list(events)

    def arrays(self):
        return LY.replicate(self.dp, self.M)

    def fault_array(self, dt=DT):
        return LY.fault_array(self.faults, dt, self.events)


def psse_case(cases, raw, dyr, alpha=0.5, drop_dyr_gens=()):
    dyr_recs = [r for r in cases["dyr"][dyr] if not (r[1].strip("'") in ("GENROU", "GENSAL") and int(r[0]) in drop_dyr_gens)]
    ps = psse.from_records(cases["raw"][raw], dyr_recs, load_alpha=alpha)
    dp = M.initialize_dynamics(ps)
    return ps, dp


def case9_system(known):
    c9 = known["case9"]
    buses = [M.Bus(int(b[0]), b[1], int(b[2]), float(b[3]), float(b[4]), float(b[5])) for b in c9["buses"]]
    bm = {b.i: k for k, b in enumerate(buses)}
    gens = [M.Gen(bm[int(g[0])], g[1], float(g[2]), float(g[3]), float(g[4])) for g in c9["gens"]]
    loads = [M.Load(bm[int(l[0])], l[1], float(l[2]), float(l[3])) for l in c9["loads"]]
    brs = [M.Branch(bm[int(x[0])], bm[int(x[1])], x[2], *map(float, x[3:8])) for x in c9["branches"]]
    ps = M.PowerSystem(c9["baseMVA"], buses, gens, loads, brs, [], bm)
    M.build_network(ps)
    return ps


def run_oracle(orc, case, nsteps, solver=0, itermax=50, dt=DT, z0=None, nthreads=1):
    z, u, p = case.arrays()
    if z0 is not None:
        z = np.ascontiguousarray(z0)
    fa, nf = case.fault_array(dt)
    return orc.integrate(case.PA, z, u, p, fa, nf, dt, nsteps, solver=solver, itermax=itermax,
                         nthreads=nthreads)


def synthetic_case(name, M_):
    w = synthetic.WORKLOADS[name]()
    faults = (w.faults * ((M_ + len(w.faults) - 1) // len(w.faults)))[:M_]
    return Case(w.ps, w.dp, faults, M_), w
