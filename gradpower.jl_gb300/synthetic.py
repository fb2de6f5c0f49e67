"""Seeded synthetic grids for the five benchmark workloads of this path.

The reference ships no large cases (its 2,000- and 70,000-bus files are not in
the repository), so every workload is generated here from a seed, in the
reference's own data model (buses, generators, loads with the stored Q
negated, branches) and then taken through the same setup as a PSS/E case:
`build_network`, `runpf_inplace`, `set_dynamics`, `initialize_dynamics`.

Workloads (sizes and parameter distributions as the benchmark definition
states them; choices it leaves open are recorded in `Workload.notes`):

* ``two_bus``    — 2-bus GENROU + IEESGO, fault on bus 2, 10 s, M=1.
* ``ring39``     — 39-bus ring + 7 chords, 10 GENROU+SEXS+TGOV1, 19 ZIP loads,
                   one seeded fault bus per scenario, 1 s, M=64.
* ``planar2k``   — 2,000-bus planar graph (mean degree 2.7), 400 machines
                   (GENROU/GENSAL, SEXS/ESDC1A, IEEEST on 25 %, TGOV1/IEESGO),
                   ZIP loads on 60 % of buses, 2 s, M=256.
* ``planar2k_adj`` — the same grid, 3 s, M=128.
* ``planar70k``  — 70,000-bus planar graph, 5,000 machines, ZIP loads on
                   55 % of buses, faults on top-decile-degree buses, 1 s, M=8.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List

import numpy as np
import scipy.sparse as sp
from scipy.sparse.csgraph import minimum_spanning_tree, connected_components

from . import model as M


@dataclass
class Workload:
    name: str
    ps: M.PowerSystem
    dp: M.DynamicProblem
    n_scenarios: int
    tf: float
    dt: float
    faults: List[List[M.ContingencyEvent]]      # per scenario
    notes: List[str] = field(default_factory=list)


# ---------------------------------------------------------------------------
# parameter draws
# ---------------------------------------------------------------------------

GENROU_BASE = dict(x_d=1.8, x_q=1.7, x_dp=0.3, x_qp=0.55, x_ddp=0.25, xl=0.2,
                   T_d0p=6.0, T_q0p=0.5, T_d0dp=0.03, T_q0dp=0.05, S1=0.09, S2=0.38)


def _genrou(rng, bus, ident, H_range, spread, salient=False):
    b = GENROU_BASE
    if spread > 0:
        # one factor for the whole reactance chain keeps x_d > x_dp > x_ddp > xl
        fx = rng.uniform(1 - spread, 1 + spread)
        ft = rng.uniform(1 - spread, 1 + spread, size=4)
        fs = rng.uniform(1 - spread, 1 + spread)
    else:
        fx, ft, fs = 1.0, np.ones(4), 1.0
    H = rng.uniform(*H_range)
    kw = dict(x_d=b["x_d"] * fx, x_q=b["x_q"] * fx, x_dp=b["x_dp"] * fx,
              x_qp=b["x_qp"] * fx, x_ddp=b["x_ddp"] * fx, xl=b["xl"] * fx,
              H=H, D=0.0,
              T_d0p=b["T_d0p"] * ft[0], T_q0p=b["T_q0p"] * ft[1],
              T_d0dp=b["T_d0dp"] * ft[2], T_q0dp=b["T_q0dp"] * ft[3],
              S1=b["S1"] * fs, S2=b["S2"] * fs)
    if salient:
        return M.Genrou.gensal(bus, ident, kw["x_d"], kw["x_q"], kw["x_dp"], kw["x_ddp"],
                               kw["xl"], kw["H"], kw["D"], kw["T_d0p"], kw["T_d0dp"],
                               kw["T_q0dp"], kw["S1"], kw["S2"])
    return M.Genrou(bus, ident, **kw)


def _ieesgo(rng, bus, ident):
    T = rng.uniform(0.05, 0.5, size=6)
    return M.IEESGO(bus, ident, *T, 20.0, 0.5, 0.5, 1.2, 0.0)


def _tgov1(bus, ident):
    return M.TGOV1(bus, ident, 0.05, 0.5, 1.2, 0.0, 1.0, 2.0, 0.0)


def _sexs(bus, ident):
    return M.SEXS(bus, ident, 0.1, 10.0, 100.0, 0.05, -5.0, 5.0)


def _esdc1a(bus, ident):
    # KA=400, TA=0.02, KF=0.03, TF=1, KE=1, TE=0.8, TR unused, no saturation
    return M.ESDC1A(bus, ident, 400.0, 0.02, 0.03, 1.0, 1.0, 0.8, 0.0, 0.0, 0.0)


def _ieeest(bus, ident):
    # unity 2nd-order filters, one lead-lag pair, washout 1 s, KS=5
    return M.IEEEST(bus, ident, 1, 0, 0.05, 0.005, 0.05, 0.005, 0.05, 0.005,
                    0.15, 0.05, 0.15, 0.05, 1.0, 1.0, 5.0, 0.1, -0.1, 0.0, 0.0)


# ---------------------------------------------------------------------------
# graphs
# ---------------------------------------------------------------------------

def ring_with_chords(rng, n, n_chords):
    edges = {(i, (i + 1) % n) for i in range(n)}
    edges = {tuple(sorted(e)) for e in edges}
    while len(edges) < n + n_chords:
        a, b = rng.choice(n, size=2, replace=False)
        e = tuple(sorted((int(a), int(b))))
        if abs(e[0] - e[1]) in (1, n - 1):
            continue
        edges.add(e)
    return sorted(edges), None


def planar_graph(rng, n, mean_degree=2.7):
    """Connected planar graph on random points: the Euclidean minimum
    spanning tree of the Delaunay triangulation plus the shortest remaining
    Delaunay edges until the edge count is round(mean_degree * n / 2)."""
    from scipy.spatial import Delaunay
    pts = rng.random((n, 2))
    tri = Delaunay(pts)
    s = tri.simplices
    e = np.concatenate([s[:, [0, 1]], s[:, [1, 2]], s[:, [0, 2]]])
    e.sort(axis=1)
    e = np.unique(e, axis=0)
    length = np.linalg.norm(pts[e[:, 0]] - pts[e[:, 1]], axis=1)
    G = sp.coo_matrix((length + 1e-12, (e[:, 0], e[:, 1])), shape=(n, n)).tocsr()
    T = minimum_spanning_tree(G).tocoo()
    tree = {(min(a, b), max(a, b)) for a, b in zip(T.row.tolist(), T.col.tolist())}
    target = int(round(mean_degree * n / 2))
    order = np.argsort(length, kind="stable")
    edges = set(tree)
    for k in order:
        if len(edges) >= target:
            break
        edges.add((int(e[k, 0]), int(e[k, 1])))
    edges = sorted(edges)
    A = sp.coo_matrix((np.ones(len(edges)), ([a for a, _ in edges], [b for _, b in edges])),
                      shape=(n, n))
    assert connected_components(A, directed=False)[0] == 1
    return edges, pts


# ---------------------------------------------------------------------------
# assembly
# ---------------------------------------------------------------------------

def _build(name, rng, n_bus, edges, gen_buses, load_buses, load_p, machines,
           b_range, slack_v=1.0, pv_v=(1.0, 1.04), M_scen=1, tf=1.0,
           fault_buses=None, rf_range=(0.01, 0.2), ton=0.1, toff=0.2,
           load_alpha=0.4, fixed_faults=None, notes=(), load_q=None,
           branch_params=None):
    buses = []
    gset = set(gen_buses)
    for i in range(n_bus):
        if i == gen_buses[0]:
            buses.append(M.Bus(i + 1, "B%d" % (i + 1), M.SLACK, 345.0, slack_v, 0.0))
        elif i in gset:
            buses.append(M.Bus(i + 1, "B%d" % (i + 1), M.PV, 345.0,
                               float(rng.uniform(*pv_v)), 0.0))
        else:
            buses.append(M.Bus(i + 1, "B%d" % (i + 1), M.PQ, 345.0, 1.0, 0.0))
    branches = []
    for k, (a, b) in enumerate(edges):
        if branch_params is not None:
            r, x, sh = branch_params[k]
        else:
            r = rng.uniform(0.001, 0.01)
            x = rng.uniform(0.01, 0.1)
            sh = rng.uniform(*b_range)
        branches.append(M.Branch(a, b, "1", r, x, sh))
    if load_q is None:
        load_q = 0.3 * np.asarray(load_p)
    loads = [M.Load(bus, "1", float(pl), -float(ql))
             for bus, pl, ql in zip(load_buses, load_p, load_q)]
    # Dispatch: every load is served by its nearest generator (multi-source
    # breadth-first search over the branch graph), so flows stay local.
    owner = np.full(n_bus, -1, dtype=np.int64)
    nbr = [[] for _ in range(n_bus)]
    for (a, b) in edges:
        nbr[a].append(b)
        nbr[b].append(a)
    frontier = list(gen_buses)
    for k, gb in enumerate(gen_buses):
        owner[gb] = k
    while frontier:
        nxt = []
        for u in frontier:
            for v in nbr[u]:
                if owner[v] < 0:
                    owner[v] = owner[u]
                    nxt.append(v)
        frontier = nxt
    pg = np.zeros(len(gen_buses))
    for bus, pl in zip(load_buses, load_p):
        pg[owner[bus]] += pl
    if n_bus > 100:
        # Spread the expected I^2 R losses over all machines (estimated from
        # a DC flow) so that the single slack bus does not carry them all.
        from scipy.sparse.linalg import spsolve
        inj = np.zeros(n_bus)
        for k, gb in enumerate(gen_buses):
            inj[gb] += pg[k]
        for bus, pl in zip(load_buses, load_p):
            inj[bus] -= pl
        ea = np.array([a for a, _ in edges])
        eb = np.array([b for _, b in edges])
        xs = np.array([br.x for br in branches])
        rs = np.array([br.r for br in branches])
        w = 1.0 / xs
        Lap = sp.csr_matrix((np.concatenate([w, w, -w, -w]),
                             (np.concatenate([ea, eb, ea, eb]), np.concatenate([ea, eb, eb, ea]))),
                            shape=(n_bus, n_bus))
        keep = np.arange(1, n_bus)
        th = np.zeros(n_bus)
        th[keep] = spsolve(Lap[keep][:, keep].tocsc(), inj[keep])
        flow = (th[ea] - th[eb]) / xs
        loss = rs * flow ** 2
        pg *= 1.0 + float(np.sum(loss)) / float(np.sum(load_p))
        # start the power flow from DC angles that already carry the branch
        # losses as loads at the branch ends (a solved case would carry its
        # own angles), referenced to the slack gen_buses[0]
        inj[:] = 0.0
        for k, gb in enumerate(gen_buses):
            inj[gb] += pg[k]
        for bus, pl in zip(load_buses, load_p):
            inj[bus] -= pl
        np.add.at(inj, ea, -0.5 * loss)
        np.add.at(inj, eb, -0.5 * loss)
        th = np.zeros(n_bus)
        th[keep] = spsolve(Lap[keep][:, keep].tocsc(), inj[keep])
        th -= th[gen_buses[0]]
        for i in range(n_bus):
            buses[i].v0a = float(th[i])
    gens = [M.Gen(bus, "1", float(pg[k]), 0.0, 100.0) for k, bus in enumerate(gen_buses)]
    ps = M.PowerSystem(100.0, buses, gens, loads, branches, [],
                       {i + 1: i for i in range(n_bus)})
    devices = []
    for k, bus in enumerate(gen_buses):
        devices.append(machines[k][0])
    for k in range(len(gen_buses)):
        for d in machines[k][1:]:
            if d is not None and not d.is_stabilizer:
                devices.append(d)
    for k in range(len(gen_buses)):
        for d in machines[k][1:]:
            if d is not None and d.is_stabilizer:
                devices.append(d)
    psd = M.PowerSystemDynamics(devices)
    M.build_network(ps)
    M.runpf_inplace(ps)
    M.set_dynamics(ps, psd, load_alpha=load_alpha)
    dp = M.initialize_dynamics(ps)
    faults = []
    if fixed_faults is not None:
        faults = fixed_faults
    else:
        for m in range(M_scen):
            fb = int(fault_buses[m])
            rf = float(rng.uniform(*rf_range))
            faults.append([M.ContingencyEvent(fb, rf, ton, toff)])
    return Workload(name, ps, dp, M_scen, tf, 1.0 / 120.0, faults, list(notes))


def two_bus(seed=0):
    rng = np.random.default_rng(seed)
    gen = _genrou(rng, 1, "1", (3.0, 6.0), 0.0)
    gov = _ieesgo(rng, 1, "1")
    return _build("two_bus", rng, 2, [(0, 1)], [0], [1], np.array([0.8]),
                  [[gen, gov, None, None]], (0.0, 0.0), slack_v=1.0,
                  M_scen=1, tf=10.0, load_alpha=1.0, load_q=np.array([0.3]),
                  branch_params=[(0.01, 0.1, 0.0)],
                  fixed_faults=[[M.ContingencyEvent(1, 0.2, 0.2, 0.3)]],
                  notes=["ZIP load at the reference's default alpha=1 (set_dynamics!)",
                         "slack voltage 1.0 pu"])


def ring39(seed=1, n_scenarios=64):
    rng = np.random.default_rng(seed)
    n = 39
    edges, _ = ring_with_chords(rng, n, 7)
    perm = rng.permutation(n)
    gen_buses = [int(b) for b in perm[:10]]
    load_buses = [int(b) for b in perm[10:29]]
    # The stated P ~ U[0.5, 3] pu has no power-flow solution on a 39-bus ring
    # with x ~ U[0.01, 0.1] (voltage collapse); the draw is halved.
    load_p = 0.5 * rng.uniform(0.5, 3.0, size=19)
    machines = []
    for k, bus in enumerate(gen_buses):
        g = _genrou(rng, bus + 1, "1", (3.0, 10.0), 0.2)
        machines.append([g, _tgov1(bus + 1, "1"), _sexs(bus + 1, "1"), None])
    fault_buses = rng.choice(n, size=n_scenarios, replace=n_scenarios > n)
    return _build("ring39", rng, n, edges, gen_buses, load_buses, load_p, machines,
                  (0.0, 0.4), M_scen=n_scenarios, tf=1.0, fault_buses=fault_buses,
                  notes=["load P ~ 0.5 x U[0.5, 3] pu: the unscaled draw has no power-flow "
                         "solution on this ring (voltage collapse)",
                         "ZIP split 0.4/0.3/0.3 mapped to alpha=0.4 (the reference "
                         "model has no constant-current part)",
                         "fault onset 0.1 s, cleared at 0.2 s",
                         "TGOV1 VMAX=1.2, VMIN=0, DT=0 (not enforced by the model)"])


def _planar(name, seed, n_bus, n_gen, load_frac, n_scenarios, tf, fault_mode, b_range=(0.0, 0.0),
            load_range=(0.005, 0.03), extra_notes=()):
    rng = np.random.default_rng(seed)
    edges, pts = planar_graph(rng, n_bus)
    # Machines are spread evenly: one per cell of a square grid laid over the
    # unit square (random bus inside the cell), the remaining ones at random.
    # Purely random placement leaves load pockets hundreds of buses from any
    # machine, which have no power-flow solution.
    side = int(math.floor(math.sqrt(n_gen)))
    cell = np.minimum((pts * side).astype(np.int64), side - 1)
    cid = cell[:, 0] * side + cell[:, 1]
    order = rng.permutation(n_bus)
    chosen = {}
    for b in order:
        c = int(cid[b])
        if c not in chosen:
            chosen[c] = int(b)
    gen_buses = list(chosen.values())[:n_gen]
    gset = set(gen_buses)
    rest = [int(b) for b in order if int(b) not in gset]
    gen_buses += rest[:n_gen - len(gen_buses)]
    gset = set(gen_buses)
    rest = [b for b in rest if b not in gset]
    n_load = int(round(load_frac * n_bus))
    load_buses = rest[:n_load]
    load_p = rng.uniform(*load_range, size=n_load)
    machines = []
    kinds = rng.random((n_gen, 4))
    for k, bus in enumerate(gen_buses):
        b1 = bus + 1
        g = _genrou(rng, b1, "1", (3.0, 10.0), 0.2, salient=kinds[k, 0] >= 0.6)
        exc = _sexs(b1, "1") if kinds[k, 1] < 0.5 else _esdc1a(b1, "1")
        pss = _ieeest(b1, "1") if kinds[k, 2] < 0.25 else None
        gov = _tgov1(b1, "1") if kinds[k, 3] < 0.5 else _ieesgo(rng, b1, "1")
        machines.append([g, gov, exc, pss])
    deg = np.zeros(n_bus, dtype=np.int64)
    for a, b in edges:
        deg[a] += 1
        deg[b] += 1
    if fault_mode == "high_degree":
        cut = np.quantile(deg, 0.9)
        cand = np.where(deg >= cut)[0]
        fault_buses = rng.choice(cand, size=n_scenarios, replace=n_scenarios > len(cand))
    else:
        fault_buses = rng.choice(n_bus, size=n_scenarios, replace=n_scenarios > n_bus)
    return _build(name, rng, n_bus, edges, gen_buses, load_buses, load_p, machines,
                  b_range, pv_v=(1.0, 1.0), M_scen=n_scenarios, tf=tf,
                  fault_buses=fault_buses,
                  notes=["planar graph: Delaunay MST + shortest Delaunay edges to mean degree 2.7",
                         "load P ~ U[0.005, 0.03] pu with Q = 0.3 P (per-bus size not fixed by the benchmark; "
                         "heavier loads have no power-flow solution on radial stretches of the graph)",
                         "each load is served by its nearest generator (dispatch to balance), "
                         "machines scaled up by the DC-estimated I^2 R losses",
                         "no line charging and all voltage set points 1.0 pu on the planar grids: "
                         "charging in the 39-bus range, or scattered set points between "
                         "neighbouring machines, leave the power flow without a solution",
                         "ZIP split mapped to alpha=0.4; fault onset 0.1 s, cleared at 0.2 s",
                         "IEEEST: A1=A3=A5=0.05, A2=A4=A6=0.005, T1=T3=0.15, T2=T4=0.05, "
                         "T5=T6=1, KS=5"])


def planar2k(seed=2, n_scenarios=256):
    return _planar("planar2k", seed, 2000, 400, 0.6, n_scenarios, 2.0, "random")


def planar2k_adj(seed=2, n_scenarios=128):
    w = _planar("planar2k_adj", seed, 2000, 400, 0.6, n_scenarios, 3.0, "random")
    return w


def planar70k(seed=4, n_scenarios=8):
    return _planar("planar70k", seed, 70000, 5000, 0.55, n_scenarios, 1.0, "high_degree")


def planar2k_stressed(seed=2, n_scenarios=256):
    """planar2k with four times the loads (P ~ U[0.02, 0.12] pu) and line
    charging b ~ U[0, 0.1] pu (a quarter of the 39-bus range): the heaviest
    variant of the 2,000-bus grid that keeps a power-flow solution (b up to
    0.2 also solves; 0.4 does not)."""
    w = _planar("planar2k_stressed", seed, 2000, 400, 0.6, n_scenarios, 2.0, "random", b_range=(0.0, 0.1),
                load_range=(0.02, 0.12))
    w.notes.append("stressed variant: loads x4 (U[0.02, 0.12] pu), line charging b ~ U[0, 0.1] pu")
    return w


def planar70k_charged(seed=4, n_scenarios=8):
    """planar70k with line charging b ~ U[0, 0.01] pu, the most the
    70,000-bus grid takes: b up to 0.02, or loads 1.5 times heavier, leave
    its power flow without a solution."""
    w = _planar("planar70k_charged", seed, 70000, 5000, 0.55, n_scenarios, 1.0, "high_degree",
                b_range=(0.0, 0.01))
    w.notes.append("charged variant: line charging b ~ U[0, 0.01] pu")
    return w


WORKLOADS = {
    "two_bus": two_bus,
    "ring39": ring39,
    "planar2k": planar2k,
    "planar2k_adj": planar2k_adj,
    "planar70k": planar70k,
    "planar2k_stressed": planar2k_stressed,
    "planar70k_charged": planar70k_charged,
}
