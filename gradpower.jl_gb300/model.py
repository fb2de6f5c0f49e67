"""Power-system data model and the host-once problem setup of the batched
backward-Euler Newton path.

This module restates, in Python, the reference's setup layer that runs once
before the hot loop: the network data model (GradPower.jl `src/GradPower.jl:22-63`),
the complex and realified bus admittance matrix (`src/network.jl:15-126`), the
polar Newton power flow (`src/pflow.jl:1-53,286-418`), the device models and their
parameter vectors (`src/generators.jl`, `src/governors.jl`, `src/exciters.jl`,
`src/stabilizers.jl`, `src/loads.jl`, `src/static_gen.jl`), `set_dynamics!`
(`src/GradPower.jl:297-447`), the trait-driven control wiring
(`src/coupling.jl:154-256`), the generator clusters with their
cluster-contiguous state ordering (`src/clusters.jl:73-319`) and the device
initialisation (`src/dynamics.jl:8-250`).

Everything here is setup: it produces the state vector z0, the control vector
u0, the parameter vector p and the pointer tables that the C-ABI library
(`libgradpower_gb300.so`) consumes.  All indices are 0-based.  Unlike the
reference, `alg_ptr` is stored as an absolute z index (the reference stores it
relative to `diff_dim`), so every pointer below addresses z directly.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

TWOPI60 = 2.0 * math.pi * 60.0

# Bus types (PSS/E convention, `src/static_gen.jl` / `src/kernels/static_gen.jl`).
PQ, PV, SLACK = 1, 2, 3


# ---------------------------------------------------------------------------
# Network data model (src/GradPower.jl:22-63)
# ---------------------------------------------------------------------------

@dataclass
class Bus:
    i: int            # external bus number
    id: str
    type: int         # 1 PQ, 2 PV, 3 slack
    baseKV: float
    v0m: float
    v0a: float        # radians


@dataclass
class Gen:
    bus: int          # internal 0-based bus index
    id: str
    psch: float       # pu on system base
    qsch: float
    mbase: float
    status: bool = True


@dataclass
class Load:
    bus: int
    id: str
    pd: float
    qd: float         # stored NEGATED, as raw_to_grad does (src/parse.jl:384)


@dataclass
class Branch:
    fr: int
    to: int
    id: str
    r: float
    x: float
    sh: float
    tap: float = 0.0
    shift: float = 0.0


@dataclass
class Shunt:
    bus: int
    id: str
    gsh: float
    bsh: float


@dataclass
class ContingencyEvent:
    """Three-phase bus fault (src/GradPower.jl:117-128).  `bus` is the
    internal 0-based bus index; `rfault` the fault resistance in pu."""
    bus: int
    rfault: float
    ton: float
    toff: float
    status: bool = False


@dataclass
class TripLineEvent:
    """Line trip (src/GradPower.jl:148-167): the line's admittance terms
    leave Ybus at ton and come back at toff (inf: permanent).  Buses are
    internal 0-based indices; the y terms are complex."""
    from_bus: int
    to_bus: int
    ton: float
    toff: float
    yff: complex
    yft: complex
    ytf: complex
    ytt: complex


@dataclass
class DisconnectDeviceEvent:
    """Device disconnection (src/GradPower.jl:131-146): the device's online
    flag is cleared at ton for the rest of the run.  device_idx is the
    0-based index into PowerSystemDynamics.devices."""
    device_idx: int
    ton: float


def create_trip_line_event(ps: "PowerSystem", from_bus_ext: int, to_bus_ext: int, ton: float,
                           toff: float = math.inf) -> TripLineEvent:
    """The branch between two buses given by their external (PSS/E) numbers
    and its admittance terms, as Ybus holds them (create_trip_line_event,
    src/GradPower.jl:500-543)."""
    fr_i = ps.busmap[from_bus_ext] if ps.busmap else from_bus_ext
    to_i = ps.busmap[to_bus_ext] if ps.busmap else to_bus_ext
    for br in ps.branches:
        if (br.fr, br.to) in ((fr_i, to_i), (to_i, fr_i)):
            return trip_branch_event(br, ton, toff)
    raise ValueError("no branch between buses %d and %d" % (from_bus_ext, to_bus_ext))


def trip_branch_event(br: "Branch", ton: float, toff: float = math.inf) -> TripLineEvent:
    """TripLineEvent of one branch (its Ybus terms, as build_network adds
    them)."""
    tap, shift = br.tap, br.shift
    if tap > 0.0:
        tpsh = tap * np.exp(1j * math.pi / 180.0 * shift)
    else:
        tpsh = 1.0 + 0.0j
        tap = 1.0
    y = 1.0 / complex(br.r, br.x)
    return TripLineEvent(br.fr, br.to, ton, toff,
                         y / (tap * tap) + 1j * 0.5 * br.sh, -y / np.conj(tpsh), -y / tpsh,
                         y + (1j * 0.5 * br.sh) / (tap * tap))


# ---------------------------------------------------------------------------
# Device models.  Sizes follow the reference constructors; parameter
# vectors follow each type's `fill_pvec!`.
# ---------------------------------------------------------------------------

def normalize_id(s: str) -> str:
    """Strip apostrophes and spaces from a PSS/E id (src/coupling.jl:40)."""
    return s.replace("'", "").replace(" ", "").strip()


class Device:
    kind = "device"
    diff_size = 0
    alg_size = 0
    ctrl_size = 0
    par_size = 0
    is_generator = False
    is_governor = False
    is_exciter = False
    is_stabilizer = False

    def set_ratio(self, ratio: float) -> None:
        pass

    def pvec(self) -> List[float]:
        raise NotImplementedError


class Genrou(Device):
    """GENROU round-rotor machine (src/generators.jl:1-34, 111-137).
    GENSAL maps onto it with x_qp = x_dp, T_q0p = T_d0p (src/generators.jl:41-66)."""
    kind = "genrou"
    diff_size, alg_size, ctrl_size, par_size = 6, 4, 2, 14
    is_generator = True

    def __init__(self, bus, id, x_d, x_q, x_dp, x_qp, x_ddp, xl, H, D,
                 T_d0p, T_q0p, T_d0dp, T_q0dp, S1=0.0, S2=0.0):
        self.bus, self.id = bus, id
        self.x_d, self.x_q, self.x_dp, self.x_qp = x_d, x_q, x_dp, x_qp
        self.x_ddp, self.xl, self.H, self.D = x_ddp, xl, H, D
        self.T_d0p, self.T_q0p, self.T_d0dp, self.T_q0dp = T_d0p, T_q0p, T_d0dp, T_q0dp
        self.S1, self.S2 = S1, S2
        self.e_fd0 = 0.0

    @classmethod
    def gensal(cls, bus, id, x_d, x_q, x_dp, x_ddp, xl, H, D, T_d0p, T_d0dp,
               T_q0dp, S1=0.0, S2=0.0):
        return cls(bus, id, x_d, x_q, x_dp, x_dp, x_ddp, xl, H, D, T_d0p, T_d0p,
                   T_d0dp, T_q0dp, S1, S2)

    def set_ratio(self, ratio):
        for a in ("x_d", "x_q", "x_dp", "x_qp", "x_ddp", "xl"):
            setattr(self, a, getattr(self, a) * (1.0 / ratio))
        self.H *= ratio
        self.D *= ratio

    def pvec(self):
        return [self.x_d, self.x_q, self.x_dp, self.x_qp, self.x_ddp, self.xl,
                self.H, self.D, self.T_d0p, self.T_q0p, self.T_d0dp,
                self.T_q0dp, self.S1, self.S2]


class IEESGO(Device):
    """IEEE standard steam governor (src/governors.jl:1-60)."""
    kind = "ieesgo"
    diff_size, alg_size, ctrl_size, par_size = 5, 1, 1, 12
    is_governor = True

    def __init__(self, bus, id, T1, T2, T3, T4, T5, T6, K1, K2, K3, pmax, pmin):
        self.bus, self.id = bus, id
        self.T1, self.T2, self.T3, self.T4, self.T5, self.T6 = T1, T2, T3, T4, T5, T6
        self.K1, self.K2, self.K3, self.pmax, self.pmin = K1, K2, K3, pmax, pmin
        self.pref = 0.0

    def pvec(self):
        return [self.T1, self.T2, self.T3, self.T4, self.T5, self.T6, self.K1,
                self.K2, self.K3, self.pmax, self.pmin, self.pref]


class TGOV1(Device):
    """TGOV1 steam turbine-governor (src/governors.jl:140-200)."""
    kind = "tgov1"
    diff_size, alg_size, ctrl_size, par_size = 2, 1, 1, 8
    is_governor = True

    def __init__(self, bus, id, R, T1, VMAX, VMIN, T2, T3, DT):
        self.bus, self.id = bus, id
        self.R, self.T1, self.VMAX, self.VMIN = R, T1, VMAX, VMIN
        self.T2, self.T3, self.DT = T2, T3, DT
        self.pref = 0.0

    def set_ratio(self, ratio):
        self.R /= ratio
        self.VMAX /= ratio
        self.VMIN /= ratio
        self.DT *= ratio

    def pvec(self):
        return [self.R, self.T1, self.VMAX, self.VMIN, self.T2, self.T3, self.DT,
                self.pref]


class SEXS(Device):
    """Simplified excitation system (src/exciters.jl:317-359)."""
    kind = "sexs"
    diff_size, alg_size, ctrl_size, par_size = 2, 0, 1, 7
    is_exciter = True

    def __init__(self, bus, id, TA_TB, TB, K, TE, EMIN, EMAX):
        self.bus, self.id = bus, id
        self.TA_TB, self.TB, self.K, self.TE = TA_TB, TB, K, TE
        self.EMIN, self.EMAX = EMIN, EMAX
        self.vref = 0.0

    def pvec(self):
        return [self.TA_TB, self.TB, self.K, self.TE, self.EMIN, self.EMAX, self.vref]


def esdc1a_sat_coefficients(E1, SE1, E2, SE2):
    """Quadratic exciter saturation fit (src/exciters.jl:39-50)."""
    if E1 <= 0.0 or E2 <= 0.0 or SE1 <= 0.0 or SE2 <= 0.0:
        return 0.0, 0.0
    a = math.sqrt(SE1 * E1 / (SE2 * E2))
    if a == 1.0:
        return 0.0, 0.0
    sat_a = E2 - (E1 - E2) / (a - 1.0)
    sat_b = SE2 * E2 * (a - 1.0) ** 2 / (E1 - E2) ** 2
    return sat_a, sat_b


class ESDC1A(Device):
    """Reduced ESDC1A DC exciter (src/exciters.jl:3-88); Ae/Be hold the
    quadratic saturation coefficients sat_a/sat_b."""
    kind = "esdc1a"
    diff_size, alg_size, ctrl_size, par_size = 3, 0, 0, 10
    is_exciter = True

    def __init__(self, bus, id, Ka, Ta, Kf, Tf, Ke, Te, Tr, Ae, Be):
        self.bus, self.id = bus, id
        self.Ka, self.Ta, self.Kf, self.Tf, self.Ke, self.Te = Ka, Ta, Kf, Tf, Ke, Te
        self.Tr, self.Ae, self.Be = Tr, Ae, Be
        self.vref = 0.0

    def pvec(self):
        return [self.Ka, self.Ta, self.Kf, self.Tf, self.Ke, self.Te, self.Tr,
                self.Ae, self.Be, self.vref]


class IEEEST(Device):
    """IEEEST power system stabiliser, MODE=1 (src/stabilizers.jl:57-160).
    Zero time constants are clamped to 1e-3 as the reference's parser does."""
    kind = "ieeest"
    diff_size, alg_size, ctrl_size, par_size = 7, 1, 1, 19
    is_stabilizer = True

    def __init__(self, bus, id, MODE, BUSR, A1, A2, A3, A4, A5, A6, T1, T2, T3,
                 T4, T5, T6, KS, LSMAX, LSMIN, VCU, VCL):
        if MODE != 1:
            raise ValueError("IEEEST MODE=%d not supported; only MODE=1" % MODE)
        eps = 0.001
        c = lambda v: eps if v == 0.0 else v
        self.bus, self.id, self.MODE, self.BUSR = bus, id, MODE, BUSR
        self.A1, self.A2, self.A3, self.A4, self.A5, self.A6 = map(c, (A1, A2, A3, A4, A5, A6))
        self.T1, self.T2, self.T3, self.T4, self.T5, self.T6 = map(c, (T1, T2, T3, T4, T5, T6))
        self.KS, self.LSMAX, self.LSMIN, self.VCU, self.VCL = KS, LSMAX, LSMIN, VCU, VCL

    def pvec(self):
        return [self.A1, self.A2, self.A3, self.A4, self.A5, self.A6, self.T1,
                self.T2, self.T3, self.T4, self.T5, self.T6, self.KS, self.LSMAX,
                self.LSMIN, self.VCU, self.VCL, float(self.MODE), float(self.BUSR)]


class ZIPLoad(Device):
    """Static load as a Z + P current injection (src/loads.jl:1-40).  Only
    the constant-impedance share alpha and the constant-power share 1-alpha
    enter the equations; beta and gamma are carried but unused, as in the
    reference kernel (src/kernels/zipload.jl:33-85)."""
    kind = "zipload"
    diff_size, alg_size, ctrl_size, par_size = 0, 0, 0, 9

    def __init__(self, bus, id, pinj, qinj, alpha=1.0, beta=0.0, gamma=0.0,
                 weight=1.0, v0mag=1.0, yreal=0.0, yimag=0.0):
        self.bus, self.id = bus, id          # bus: internal index
        self.pinj, self.qinj = pinj, qinj
        self.alpha, self.beta, self.gamma, self.weight = alpha, beta, gamma, weight
        self.v0mag, self.yreal, self.yimag = v0mag, yreal, yimag

    def pvec(self):
        return [self.pinj, self.qinj, self.alpha, self.beta, self.gamma,
                self.weight, self.v0mag, self.yreal, self.yimag]


class StaticGenerator(Device):
    """Stand-in injection for a static generator without a machine model
    (src/static_gen.jl).  PQ: no states; PV: alg q; SLACK: alg p, q."""
    kind = "static_gen"
    diff_size, ctrl_size, par_size = 0, 0, 4

    def __init__(self, bus, bus_type, gen_idxs, vset, aset):
        self.bus = bus                       # external bus number
        self.id = "sg"
        self.bus_type = bus_type
        self.gen_idxs = list(gen_idxs)
        self.vset, self.aset = vset, aset
        self.p0 = 0.0
        self.q0 = 0.0
        self.alg_size = 1 if bus_type == PV else (2 if bus_type == SLACK else 0)

    def pvec(self):
        return [self.p0, self.q0, self.vset, self.aset]


# ---------------------------------------------------------------------------
# Power system + network (src/GradPower.jl:197-213, src/network.jl)
# ---------------------------------------------------------------------------

@dataclass
class PowerSystem:
    baseMVA: float
    buses: List[Bus]
    gens: List[Gen]
    loads: List[Load]
    branches: List[Branch]
    shunts: List[Shunt]
    busmap: Dict[int, int] = field(default_factory=dict)
    ybus: Optional[sp.csr_matrix] = None       # complex, n_bus x n_bus
    adjacency: Optional[List[List[int]]] = None
    dynamic: Optional["PowerSystemDynamics"] = None

    @property
    def nbus(self):
        return len(self.buses)


def build_network(ps: PowerSystem) -> None:
    """Adjacency lists and complex Ybus, restating `adjacency_list` and
    `create_ybus_complex` (src/network.jl:15-85), including the reference's
    placement of the tap-scaled half charging on the `to` end."""
    n = ps.nbus
    adj = [set() for _ in range(n)]
    for br in ps.branches:
        adj[br.fr].add(br.to)
        adj[br.to].add(br.fr)
    ps.adjacency = [sorted(a) for a in adj]

    entries: Dict[tuple, complex] = {}

    def add(i, j, v):
        entries[(i, j)] = entries.get((i, j), 0.0) + v

    for br in ps.branches:
        tap, shift = br.tap, br.shift
        if tap > 0.0:
            tpsh = tap * np.exp(1j * math.pi / 180.0 * shift)
        else:
            tpsh = 1.0 + 0.0j
            tap = 1.0
        y = 1.0 / complex(br.r, br.x)
        fr, to = br.fr, br.to
        add(fr, fr, y / (tap * tap))
        add(to, to, y)
        add(fr, to, -y / np.conj(tpsh))
        add(to, fr, -y / tpsh)
        add(to, to, (1j * 0.5 * br.sh) / (tap * tap))
        add(fr, fr, 1j * 0.5 * br.sh)
    for sh in ps.shunts:
        add(sh.bus, sh.bus, complex(sh.gsh, sh.bsh))
    if entries:
        keys = np.array(list(entries.keys()), dtype=np.int64)
        vals = np.array(list(entries.values()), dtype=np.complex128)
        Y = sp.csr_matrix((vals, (keys[:, 0], keys[:, 1])), shape=(n, n))
    else:
        Y = sp.csr_matrix((n, n), dtype=np.complex128)
    Y.sort_indices()
    ps.ybus = Y


def realify_ybus(Y: sp.spmatrix) -> sp.csc_matrix:
    """Realified admittance [g -b; b g] per complex entry (src/network.jl:87-126)."""
    Y = sp.coo_matrix(Y)
    r, c, v = Y.row, Y.col, Y.data
    rows = np.concatenate([2 * r, 2 * r + 1, 2 * r, 2 * r + 1])
    cols = np.concatenate([2 * c, 2 * c + 1, 2 * c + 1, 2 * c])
    vals = np.concatenate([v.real, v.real, -v.imag, v.imag])
    n = Y.shape[0]
    return sp.csc_matrix((vals, (rows, cols)), shape=(2 * n, 2 * n))


# ---------------------------------------------------------------------------
# Power flow (src/pflow.jl)
# ---------------------------------------------------------------------------

def _pf_injections(Y, vm, va):
    V = vm * np.exp(1j * va)
    S = V * np.conj(Y @ V)
    return S.real, S.imag


def runpf(ps: PowerSystem, tol: float = 1e-13, maxiter: int = 50):
    """Polar Newton power flow on the reference's mismatch equations
    (`resfun!`, src/pflow.jl:3-53): unknowns are |V| at PQ buses and the
    angle at PQ and PV buses; specified injections are generator output
    minus load, with the stored (negated) load Q added as the reference does.
    Returns (vm, va, p_inj, q_inj) at the solution."""
    n = ps.nbus
    btype = np.array([b.type for b in ps.buses])
    vm = np.array([b.v0m for b in ps.buses], dtype=np.float64)
    va = np.array([b.v0a for b in ps.buses], dtype=np.float64)
    pinj = np.zeros(n)
    qinj = np.zeros(n)
    for g in ps.gens:
        pinj[g.bus] += g.psch
        qinj[g.bus] += g.qsch
    for l in ps.loads:
        pinj[l.bus] -= l.pd
        qinj[l.bus] += l.qd
    pq = np.where(btype == PQ)[0]
    pqv = np.where((btype == PQ) | (btype == PV))[0]
    Y = ps.ybus.tocsr()
    for it in range(maxiter):
        P, Q = _pf_injections(Y, vm, va)
        F = np.concatenate([Q[pq] - qinj[pq], P[pqv] - pinj[pqv]])
        if F.size == 0 or np.max(np.abs(F)) < tol:
            break
        V = vm * np.exp(1j * va)
        Ibus = Y @ V
        diagV = sp.diags(V)
        diagVn = sp.diags(V / vm)
        dS_dVm = (diagV @ (Y @ diagVn).conj() + sp.diags(np.conj(Ibus)) @ diagVn).tocsr()
        dS_dVa = (1j * diagV @ (sp.diags(Ibus) - Y @ diagV).conj()).tocsr()
        J11 = dS_dVm[pq][:, pq].imag
        J12 = dS_dVa[pq][:, pqv].imag
        J21 = dS_dVm[pqv][:, pq].real
        J22 = dS_dVa[pqv][:, pqv].real
        J = sp.bmat([[J11, J12], [J21, J22]], format="csc")
        dx = spla.spsolve(J, -F)
        npq = len(pq)
        # backtracking on ||F|| keeps flat starts of large synthetic grids
        # inside the basin; a full step is taken whenever it reduces ||F||
        f0 = np.linalg.norm(F)
        lam = 1.0
        while True:
            vm_t = vm.copy(); va_t = va.copy()
            vm_t[pq] += lam * dx[:npq]
            va_t[pqv] += lam * dx[npq:]
            Pt, Qt = _pf_injections(Y, vm_t, va_t)
            Ft = np.concatenate([Qt[pq] - qinj[pq], Pt[pqv] - pinj[pqv]])
            if np.linalg.norm(Ft) < f0 or lam < 1e-3:
                break
            lam *= 0.5
        vm, va = vm_t, va_t
    else:
        raise RuntimeError("power flow did not converge")
    P, Q = _pf_injections(Y, vm, va)
    return vm, va, P, Q


def power_flow_problem(ps: PowerSystem):
    """The power flow of ps as a problem of the library's Newton step: every
    generator as a StaticGenerator stand-in (PV: q unknown and |V| = vset;
    slack: p and q unknown and V fixed; PQ: fixed injection) and every load
    as a constant-power ZIPLoad (alpha = 0).  These are the mismatch
    equations of `resfun!` (src/pflow.jl:3-53) in current-injection form, so
    the root is the power-flow solution.  Returns (ps_pf, dp_pf): ps_pf
    shares ps's network; dp_pf starts at ps's bus voltages."""
    ps2 = PowerSystem(ps.baseMVA, ps.buses, ps.gens, ps.loads, ps.branches, ps.shunts, dict(ps.busmap),
                      ps.ybus, ps.adjacency)
    psd = PowerSystemDynamics([])
    set_dynamics(ps2, psd, add_loads=True, add_static_gen_stubs=True, load_alpha=0.0)
    ps2.dynamic = psd
    return ps2, initialize_dynamics(ps2)


def runpf_inplace(ps: PowerSystem, **kw) -> None:
    """Write the power-flow solution back into the buses and generators,
    restating `runpf!` (src/pflow.jl:375-418): PV buses split the computed
    Q evenly over their generators, the slack bus splits P and Q.  The
    generator output is the computed injection minus the stored load terms,
    exactly as the reference computes it."""
    vm, va, P, Q = runpf(ps, **kw)
    apply_pf_solution(ps, vm, va, P, Q)


def apply_pf_solution(ps: PowerSystem, vm, va, P=None, Q=None) -> None:
    """The write-back half of runpf_inplace for a solution found elsewhere
    (the GPU power flow): bus voltages, then the generator outputs from the
    bus injections (computed from V when P, Q are not given)."""
    vm = np.asarray(vm, dtype=np.float64)
    va = np.asarray(va, dtype=np.float64)
    if P is None or Q is None:
        P, Q = _pf_injections(ps.ybus.tocsr(), vm, va)
    for i, b in enumerate(ps.buses):
        b.v0m = float(vm[i])
        b.v0a = float(va[i])
    sgen_p = P.copy()
    sgen_q = Q.copy()
    for l in ps.loads:
        sgen_p[l.bus] -= l.pd
        sgen_q[l.bus] -= l.qd
    bus_to_gen: List[List[int]] = [[] for _ in range(ps.nbus)]
    for gi, g in enumerate(ps.gens):
        bus_to_gen[g.bus].append(gi)
    for i, b in enumerate(ps.buses):
        ng = len(bus_to_gen[i])
        if b.type == PV:
            for gi in bus_to_gen[i]:
                ps.gens[gi].qsch = float(sgen_q[i] / ng)
        if b.type == SLACK:
            for gi in bus_to_gen[i]:
                ps.gens[gi].psch = float(sgen_p[i] / ng)
                ps.gens[gi].qsch = float(sgen_q[i] / ng)


# ---------------------------------------------------------------------------
# Dynamics container, set_dynamics!, clusters
# ---------------------------------------------------------------------------

@dataclass
class DeviceRecord:
    dtype: Device
    bus: int = -1            # internal bus index
    gen: int = -1            # index into ps.gens (generators, and propagated to controllers)
    diff_ptr: int = -1       # absolute z index of the first diff state
    alg_ptr: int = -1        # absolute z index of the first alg state
    ctrl_ptr: int = -1       # index into u of the first ctrl slot
    par_ptr: int = -1        # index into p of the first parameter
    online: bool = True


@dataclass
class Cluster:
    """A generator with its governor, exciter and stabiliser
    (src/clusters.jl:16-28).  Device fields are indices into
    `PowerSystemDynamics.devices` (-1 = absent)."""
    gen: int
    gov: int
    exc: int
    pss: int
    bus: int
    d_k: int
    a_k: int
    w_size: int
    w_start: int = -1
    trivial: bool = False


class PowerSystemDynamics:
    def __init__(self, devices: List[Device]):
        self.devices: List[DeviceRecord] = [DeviceRecord(d) for d in devices]
        self.events: List[ContingencyEvent] = []
        self.uvec_idx: Optional[np.ndarray] = None
        self.clusters: List[Cluster] = []
        self.type_groups = []
        self.diff_dim = 0
        self.alg_dim = 0
        self.ctrl_dim = 0
        self.par_dim = 0
        self.is_diff: Optional[np.ndarray] = None

    def add_event(self, ev: ContingencyEvent):
        self.events.append(ev)

    def of_kind(self, kind: str) -> List[int]:
        return [i for i, d in enumerate(self.devices) if d.dtype.kind == kind]


def _attach_target_class(dev: Device):
    if dev.is_governor or dev.is_exciter:
        return "generator"
    if dev.is_stabilizer:
        return "exciter"
    return None


_FIND_CACHE: Dict[tuple, Dict[tuple, int]] = {}


def _find_device(devs: List[DeviceRecord], cls: str, bus, idn) -> int:
    """First device of class `cls` ('gen' or 'exc') with the given external
    bus number and normalised id, as the reference's linear scans return
    (src/coupling.jl:175-183); -1 if none."""
    key = (id(devs), len(devs), cls)
    index = _FIND_CACHE.get(key)
    if index is None:
        index = {}
        for j, c in enumerate(devs):
            d = c.dtype
            ok = d.is_generator if cls == "gen" else d.is_exciter
            if ok:
                index.setdefault((d.bus, normalize_id(d.id)), j)
        if len(_FIND_CACHE) > 64:
            _FIND_CACHE.clear()
        _FIND_CACHE[key] = index
    return index.get((bus, idn), -1)


def set_dynamics(ps: PowerSystem, psd: PowerSystemDynamics,
                 add_loads: bool = True, add_static_gen_stubs: bool = True,
                 load_alpha: float = 1.0) -> None:
    """Restates `set_dynamics!` (src/GradPower.jl:297-447): bus/generator
    matching with mbase scaling, StaticGenerator stubs for unmatched active
    generators (one per bus), one ZIPLoad per static load, control wiring
    (src/coupling.jl:154-256), clusters sorted by device-type tuple
    (src/clusters.jl:73-199) and the cluster-contiguous state ordering
    z = [w_1 .. w_Nc | (vr, vi)_bus] (src/clusters.jl:225-319)."""
    mvbase = ps.baseMVA
    devs = psd.devices
    matched = []
    gen_key: Dict[tuple, int] = {}
    for k, g in enumerate(ps.gens):
        gen_key.setdefault((g.bus, normalize_id(g.id)), k)
    for rec in devs:
        d = rec.dtype
        rec.bus = ps.busmap[d.bus]
        if d.is_generator:
            gi = gen_key.get((rec.bus, normalize_id(d.id)), -1)
            rec.gen = gi
            if gi >= 0:
                d.set_ratio(ps.gens[gi].mbase / mvbase)
                matched.append(gi)
    if add_static_gen_stubs and len(matched) != len(ps.gens):
        mset = set(matched)
        by_bus: Dict[int, List[int]] = {}
        for k, g in enumerate(ps.gens):
            if k in mset:
                continue
            by_bus.setdefault(g.bus, []).append(k)
        for b_int, gidx in by_bus.items():
            bus = ps.buses[b_int]
            sg = StaticGenerator(bus.i, int(bus.type), gidx, bus.v0m, bus.v0a)
            rec = DeviceRecord(sg, bus=b_int, gen=gidx[0])
            devs.append(rec)
    if add_loads:
        for k, l in enumerate(ps.loads):
            zl = ZIPLoad(l.bus, l.id, l.pd, l.qd, load_alpha, 0.0, 0.0, 1.0,
                         ps.buses[l.bus].v0m, 0.0, 0.0)
            # the ZIP load's `bus` is already the internal index
            devs.append(DeviceRecord(zl, bus=l.bus))
    # ctrl / par pointers in device order (add_device!, src/GradPower.jl:269-280)
    ctrl = 0
    par = 0
    for rec in devs:
        d = rec.dtype
        if d.ctrl_size:
            rec.ctrl_ptr = ctrl
        ctrl += d.ctrl_size
        rec.par_ptr = par
        par += d.par_size
    psd.ctrl_dim = ctrl
    psd.par_dim = par
    psd.diff_dim = sum(r.dtype.diff_size for r in devs)
    psd.alg_dim = sum(r.dtype.alg_size for r in devs)

    # --- clusters (src/clusters.jl:73-199) ---
    gov_of: Dict[int, int] = {}
    exc_of: Dict[int, int] = {}
    pss_of: Dict[int, int] = {}
    is_gen = lambda d: d.is_generator
    for i, rec in enumerate(devs):
        d = rec.dtype
        if d.kind in ("zipload", "static_gen") or not (d.is_governor or d.is_exciter or d.is_stabilizer):
            continue
        idn = normalize_id(d.id)
        if d.is_stabilizer:
            e = _find_device(devs, 'exc', d.bus, idn)
            if e < 0:
                continue
            g = _find_device(devs, 'gen', devs[e].dtype.bus, normalize_id(devs[e].dtype.id))
            if g >= 0:
                pss_of[g] = i
        else:
            g = _find_device(devs, 'gen', d.bus, idn)
            if g < 0:
                continue
            (gov_of if d.is_governor else exc_of)[g] = i
    raw = []
    for gi, rec in enumerate(devs):
        d = rec.dtype
        if not (d.is_generator or d.kind == "static_gen"):
            continue
        members = [gi, gov_of.get(gi, -1), exc_of.get(gi, -1), pss_of.get(gi, -1)]
        d_k = sum(devs[m].dtype.diff_size for m in members if m >= 0)
        a_k = sum(devs[m].dtype.alg_size for m in members if m >= 0)
        raw.append(Cluster(members[0], members[1], members[2], members[3], rec.bus,
                           d_k, a_k, d_k + a_k, trivial=(d.kind == "static_gen")))

    def ttuple(cl):
        return tuple(devs[m].dtype.kind for m in (cl.gen, cl.gov, cl.exc, cl.pss) if m >= 0)

    raw.sort(key=ttuple)                    # stable, like Julia's default sort
    groups = []
    for ci, cl in enumerate(raw):
        tt = ttuple(cl)
        if groups and groups[-1][0] == tt:
            groups[-1][2] = ci
        else:
            groups.append([tt, ci, ci])
    psd.type_groups = [tuple(g) for g in groups]

    # --- cluster-contiguous ordering (src/clusters.jl:225-319) ---
    pos = 0
    is_diff = []
    assigned = set()
    for cl in raw:
        cl.w_start = pos
        for m in (cl.gen, cl.gov, cl.exc, cl.pss):
            if m < 0:
                continue
            rec = devs[m]
            assigned.add(m)
            if rec.dtype.diff_size:
                rec.diff_ptr = pos
            for _ in range(rec.dtype.diff_size):
                is_diff.append(True)
                pos += 1
            if rec.dtype.alg_size:
                rec.alg_ptr = pos
            for _ in range(rec.dtype.alg_size):
                is_diff.append(False)
                pos += 1
        assert pos - cl.w_start == cl.w_size
    n_da = psd.diff_dim + psd.alg_dim
    for i, rec in enumerate(devs):
        if (rec.dtype.diff_size or rec.dtype.alg_size) and i not in assigned:
            raise ValueError("device %d (%s) belongs to no generator cluster"
                             % (i, rec.dtype.kind))
    assert pos == n_da
    psd.clusters = raw
    psd.is_diff = np.array(is_diff, dtype=bool)

    # --- control wiring (src/coupling.jl:154-256) ---
    uvec = np.full(psd.ctrl_dim, -1, dtype=np.int64)
    for i, rec in enumerate(devs):
        d = rec.dtype
        tcls = _attach_target_class(d)
        if tcls is None:
            continue
        idn = normalize_id(d.id)
        if tcls == "generator":
            t = _find_device(devs, 'gen', d.bus, idn)
        else:
            t = _find_device(devs, 'exc', d.bus, idn)
        if t < 0:
            continue
        target = devs[t]
        rec.gen = target.gen
        if d.is_governor:
            uvec[target.ctrl_ptr + 1] = rec.alg_ptr          # p_m <- governor alg[0]
            uvec[rec.ctrl_ptr] = target.diff_ptr + 4         # w   <- generator w
        elif d.is_exciter:
            off = 1 if d.kind == "sexs" else 2               # e_fd diff offset
            uvec[target.ctrl_ptr + 0] = rec.diff_ptr + off
        if d.is_stabilizer:
            g = _find_device(devs, 'gen', target.dtype.bus, normalize_id(target.dtype.id))
            if g >= 0:
                uvec[rec.ctrl_ptr] = devs[g].diff_ptr + 4
                rec.gen = devs[g].gen
    psd.uvec_idx = uvec

    # mbase scaling for controllers (src/GradPower.jl:410-416)
    for rec in devs:
        d = rec.dtype
        if (d.is_governor or d.is_exciter or d.is_stabilizer) and rec.gen >= 0:
            d.set_ratio(ps.gens[rec.gen].mbase / mvbase)
    ps.dynamic = psd


# ---------------------------------------------------------------------------
# Derived wiring helpers used by the layout export
# ---------------------------------------------------------------------------

def device_links(ps: PowerSystem):
    """Per-device cross references resolved from the wiring, as the SoA
    tables carry them (src/tables/*.jl): generator pm_idx/efd_idx, governor
    w_idx, exciter vs_idx, stabiliser w_idx.  Absent links are -1."""
    psd = ps.dynamic
    uvec = psd.uvec_idx
    devs = psd.devices
    links = {}
    pss_for_exc = {}
    for i, rec in enumerate(devs):
        d = rec.dtype
        if d.is_stabilizer:
            e = _find_device(devs, 'exc', d.bus, normalize_id(d.id))
            if e >= 0:
                pss_for_exc[e] = i
    for i, rec in enumerate(devs):
        d = rec.dtype
        if d.is_generator:
            links[i] = (int(uvec[rec.ctrl_ptr + 1]), int(uvec[rec.ctrl_ptr]))
        elif d.is_governor or d.is_stabilizer:
            links[i] = (int(uvec[rec.ctrl_ptr]), -1)
        elif d.is_exciter:
            p = pss_for_exc.get(i, -1)
            links[i] = (devs[p].alg_ptr if p >= 0 else -1, -1)
        else:
            links[i] = (-1, -1)
    return links


# ---------------------------------------------------------------------------
# Device initialisation (src/dynamics.jl:8-250)
# ---------------------------------------------------------------------------

def _genrou_sat_coefficients(s1, s2):
    """src/generators.jl:71-80, vectorised."""
    s1 = np.asarray(s1, dtype=float)
    s2 = np.asarray(s2, dtype=float)
    a_out = np.zeros_like(s1)
    b_out = np.zeros_like(s1)
    ok = (s1 > 0.0) & (s2 > 0.0)
    e1, e2 = 1.0, 1.2
    a = np.sqrt(np.where(ok, s1 * e1 / np.where(ok, s2 * e2, 1.0), 1.0))
    ok &= a != 1.0
    den = np.where(ok, a - 1.0, 1.0)
    a_out = np.where(ok, e2 - (e1 - e2) / den, 0.0)
    b_out = np.where(ok, s2 * e2 * (a - 1.0) ** 2 / (e1 - e2) ** 2, 0.0)
    return a_out, b_out


def _genrou_init_residual(x, P, pg, qg, vm, va):
    """`initialize_dynamics!(::Genrou)` (src/generators.jl:208-285), for a
    batch of machines.  x: [n,12], P: [n,14]."""
    x_d, x_q, x_dp, x_qp, x_ddp, xl, H, D = (P[:, i] for i in range(8))
    T_d0p, T_q0p, T_d0dp, T_q0dp, S1, S2 = (P[:, i] for i in range(8, 14))
    x_qdp = x_ddp
    e_qp, e_dp, phi_1d, phi_2q, w, delta, v_q, v_d, i_q, i_d, e_fd, p_m = (x[:, i] for i in range(12))
    psi_de = (x_ddp - xl) / (x_dp - xl) * e_qp + (x_dp - x_ddp) / (x_dp - xl) * phi_1d
    psi_qe = -(x_ddp - xl) / (x_qp - xl) * e_dp + (x_qp - x_ddp) / (x_qp - xl) * phi_2q
    sat_a, sat_b = _genrou_sat_coefficients(S1, S2)
    psi2 = np.sqrt(psi_de * psi_de + psi_qe * psi_qe)
    on = ~((sat_b == 0.0) | (psi2 <= sat_a) | (psi2 == 0.0))
    Se = np.where(on, sat_b * (psi2 - sat_a) ** 2 / np.where(on, psi2, 1.0), 0.0)
    f = np.empty_like(x)
    f[:, 0] = (-e_qp + e_fd - (i_d - (-x_ddp + x_dp) * (-e_qp + i_d * (x_dp - xl) + phi_1d)
                               / ((x_dp - xl) ** 2.0)) * (x_d - x_dp) - Se * psi_de) / T_d0p
    f[:, 1] = (-e_dp + (i_q - (-x_qdp + x_qp) * (e_dp + i_q * (x_qp - xl) + phi_2q)
                        / ((x_qp - xl) ** 2.0)) * (x_q - x_qp)) / T_q0p
    f[:, 2] = (e_qp - i_d * (x_dp - xl) - phi_1d) / T_d0dp
    f[:, 3] = (-e_dp - i_q * (x_qp - xl) - phi_2q) / T_q0dp
    f[:, 4] = (p_m - psi_de * i_q + psi_qe * i_d) / (2.0 * H)
    f[:, 5] = TWOPI60 * w
    f[:, 6] = i_d - ((x_ddp - xl) / (x_dp - xl) * e_qp + (x_dp - x_ddp) / (x_dp - xl) * phi_1d - v_q) / x_ddp
    f[:, 7] = i_q - (-(x_qdp - xl) / (x_qp - xl) * e_dp + (x_qp - x_qdp) / (x_qp - xl) * phi_2q + v_d) / x_qdp
    f[:, 8] = v_d - vm * np.sin(delta - va)
    f[:, 9] = v_q - vm * np.cos(delta - va)
    f[:, 10] = v_d * i_d + v_q * i_q - pg
    f[:, 11] = v_q * i_d - v_d * i_q - qg
    return f


def _genrou_initial_guess(P, p, q, vm, va):
    """`initial_guess!(::Genrou)` (src/generators.jl:159-206), vectorised."""
    x_d, x_q, x_dp, x_qp, x_ddp, xl = (P[:, i] for i in range(6))
    vt = vm * np.cos(va) + 1j * vm * np.sin(va)
    ig = (p - 1j * q) / np.conj(vt)
    delta = np.angle(vt + (1j * x_q) * ig)
    v_d = vm * np.sin(delta - va)
    v_q = vm * np.cos(delta - va)
    i_d = (p * v_d + q * v_q) / (v_d ** 2 + v_q ** 2)
    i_q = (p * v_q - q * v_d) / (v_d ** 2 + v_q ** 2)
    phi_d = v_q
    phi_q = -v_d
    e_dp = (-x_qp) * i_q - phi_q
    e_qp = x_dp * i_d + phi_d
    phi_1d = e_qp - (x_dp - xl) * i_d
    phi_2q = -e_dp - (x_qp - xl) * i_q
    e_fd = e_qp + (x_d - x_dp) * i_d
    x = np.stack([e_qp, e_dp, phi_1d, phi_2q, np.zeros_like(vm), delta, v_q, v_d,
                  i_q, i_d, e_fd, p], axis=1)
    return x


def batched_newton(fun, x0, tol=1e-13, maxiter=50):
    """Newton iteration on independent small systems (one per row of x0),
    with a central-difference Jacobian.  Stands in for the reference's
    `nlsolve(..., ftol=1e-12)` call (src/dynamics.jl:49): any converging
    method lands on the same root to rounding."""
    x = x0.copy()
    n, k = x.shape
    for it in range(maxiter):
        f = fun(x)
        err = np.max(np.abs(f), axis=1) if k else np.zeros(n)
        if n == 0 or np.all(err < tol):
            break
        J = np.empty((n, k, k))
        for j in range(k):
            h = 1e-7 * np.maximum(1.0, np.abs(x[:, j]))
            xp = x.copy(); xp[:, j] += h
            xm = x.copy(); xm[:, j] -= h
            J[:, :, j] = (fun(xp) - fun(xm)) / (2.0 * h)[:, None]
        active = err >= tol
        dx = np.zeros_like(x)
        dx[active] = np.linalg.solve(J[active], f[active][..., None])[..., 0]
        x -= dx
    f = fun(x)
    return x, np.max(np.abs(f), axis=1) if k and n else np.zeros(n)


@dataclass
class DynamicProblem:
    """z0 [n_sys], u0 [n_ctrl], p [n_par] (src/GradPower.jl:169-173)."""
    zvec: np.ndarray
    uvec: np.ndarray
    pvec: np.ndarray


def initialize_dynamics(ps: PowerSystem) -> DynamicProblem:
    """Restates `initialize_dynamics!` (src/dynamics.jl:123-250): bus
    voltages from the power flow, ZIP admittances at the solved |V|, the
    parameter vector, generator init (Newton to 1e-13), StaticGenerator
    totals, then controller init with e_fd0 passed to the exciters.  Raises
    if any device's init residual exceeds 1e-9 (src/dynamics.jl:58)."""
    psd = ps.dynamic
    devs = psd.devices
    nbus = ps.nbus
    n_da = psd.diff_dim + psd.alg_dim
    z = np.zeros(n_da + 2 * nbus)
    u = np.zeros(psd.ctrl_dim)
    p = np.zeros(psd.par_dim)
    for i, b in enumerate(ps.buses):
        z[n_da + 2 * i] = b.v0m * math.cos(b.v0a)
        z[n_da + 2 * i + 1] = b.v0m * math.sin(b.v0a)
    for rec in devs:
        d = rec.dtype
        if d.kind == "zipload":
            d.v0mag = ps.buses[rec.bus].v0m
            y = complex(d.pinj, d.qinj) / (d.v0mag ** 2.0)
            d.yreal, d.yimag = y.real, y.imag
    for rec in devs:
        p[rec.par_ptr:rec.par_ptr + rec.dtype.par_size] = rec.dtype.pvec()

    def put(rec, x):
        d = rec.dtype
        ds, as_, cs = d.diff_size, d.alg_size, d.ctrl_size
        if ds:
            z[rec.diff_ptr:rec.diff_ptr + ds] = x[:ds]
        if as_:
            z[rec.alg_ptr:rec.alg_ptr + as_] = x[ds:ds + as_]
        if cs:
            u[rec.ctrl_ptr:rec.ctrl_ptr + cs] = x[ds + as_:ds + as_ + cs]

    # generators, batched over all GENROU machines
    gi = [i for i, r in enumerate(devs) if r.dtype.is_generator]
    if gi:
        P = np.array([p[devs[i].par_ptr:devs[i].par_ptr + 14] for i in gi])
        pg = np.array([ps.gens[devs[i].gen].psch for i in gi])
        qg = np.array([ps.gens[devs[i].gen].qsch for i in gi])
        vm = np.array([ps.buses[devs[i].bus].v0m for i in gi])
        va = np.array([ps.buses[devs[i].bus].v0a for i in gi])
        x0 = _genrou_initial_guess(P, pg, qg, vm, va)
        x, err = batched_newton(lambda x: _genrou_init_residual(x, P, pg, qg, vm, va), x0)
        if np.any(err >= 1e-9):
            raise RuntimeError("GENROU init residual %g exceeds 1e-9" % err.max())
        for k, i in enumerate(gi):
            put(devs[i], x[k])
            devs[i].dtype.e_fd0 = float(x[k, 10])
    # static generators
    for rec in devs:
        d = rec.dtype
        if d.kind != "static_gen":
            continue
        d.p0 = sum(ps.gens[g].psch for g in d.gen_idxs)
        d.q0 = sum(ps.gens[g].qsch for g in d.gen_idxs)
        if d.bus_type == PV:
            z[rec.alg_ptr] = d.q0
        elif d.bus_type == SLACK:
            z[rec.alg_ptr] = d.p0
            z[rec.alg_ptr + 1] = d.q0
        p[rec.par_ptr] = d.p0
        p[rec.par_ptr + 1] = d.q0
    # exciters read e_fd0 of their machine
    for rec in devs:
        d = rec.dtype
        if d.is_exciter:
            g = _find_device(devs, 'gen', d.bus, normalize_id(d.id))
            if g >= 0:
                d.vref = devs[g].dtype.e_fd0
    # controllers
    for rec in devs:
        d = rec.dtype
        if not (d.is_governor or d.is_exciter or d.is_stabilizer):
            continue
        pp = rec.par_ptr
        pv = p[pp:pp + d.par_size]
        pg = ps.gens[rec.gen].psch if rec.gen >= 0 else 0.0
        vm = ps.buses[rec.bus].v0m
        if d.kind == "ieesgo":
            K2, K3 = pv[7], pv[8]
            pref = pg
            x = np.array([0.0, 0.0, pref, K2 * pref, K2 * K3 * pref, pg, pref])

            def res(xx, pv=pv, pg=pg):
                T1, T2, T3, T4, T5, T6, K1, K2, K3 = pv[:9]
                PF0, PLL, TP1, TP2, TP3, p_m, pref = xx
                w = 0.0
                SatP = pref - (T2 / T3) * PF0 - PLL
                return np.array([(1.0 / T1) * (K1 * w - PF0),
                                 (1 / T3) * ((1.0 - (T2 / T3)) * PF0 - PLL),
                                 (1 / T4) * (SatP - TP1),
                                 (1 / T5) * (K2 * TP1 - TP2),
                                 (1 / T6) * (K3 * TP2 - TP3),
                                 TP1 * (1 - K2) + TP2 * (1 - K3) + TP3 - p_m,
                                 p_m - pg])
            x = _solve_one(res, x)
            d.pref = float(x[6])
            p[pp + 11] = d.pref
        elif d.kind == "tgov1":
            R, T2, T3 = pv[0], pv[4], pv[5]
            x2 = pg
            x = np.array([(1.0 - T2 / T3) * x2, x2, pg, R * pg])

            def res(xx, pv=pv, pg=pg):
                R, T1, _, _, T2, T3, DT = pv[:7]
                x1, x2, p_m, pref = xx
                w = 0.0
                return np.array([(-x1 + (1.0 - T2 / T3) * x2) / T3,
                                 ((pref - w) / R - x2) / T1,
                                 x1 + (T2 / T3) * x2 - DT * w - p_m,
                                 p_m - pg])
            x = _solve_one(res, x)
            d.pref = float(x[3])
            p[pp + 7] = d.pref
        elif d.kind == "sexs":
            TA_TB, K = pv[0], pv[2]
            e_fd0 = d.vref
            vg = e_fd0 / K + vm
            x = np.array([(1.0 - TA_TB) * (vg - vm), e_fd0, vg])

            def res(xx, pv=pv, vm=vm, e_fd0=e_fd0):
                TA_TB, TB, K, TE = pv[:4]
                x1, e_fd, vref = xx
                return np.array([(-x1 + (1.0 - TA_TB) * (vref - vm)) / TB,
                                 (-e_fd + K * (x1 + TA_TB * (vref - vm))) / TE,
                                 e_fd - e_fd0])
            x = _solve_one(res, x)
            d.vref = float(x[2])
            p[pp + 6] = d.vref
        elif d.kind == "esdc1a":
            Ka, Kf, Tf, Ke, sat_a, sat_b = pv[0], pv[2], pv[3], pv[4], pv[7], pv[8]
            e_fd0 = d.vref
            sat = 0.0 if (sat_b == 0.0 or e_fd0 <= sat_a) else sat_b * (e_fd0 - sat_a) ** 2
            vr1 = Ke * e_fd0 + sat
            vr2 = -(Kf / Tf) * e_fd0
            d.vref = vm + vr1 / Ka
            p[pp + 9] = d.vref
            x = np.array([vr1, vr2, e_fd0])
        elif d.kind == "ieeest":
            x = np.zeros(9)
        put(rec, x)
    return DynamicProblem(z, u, p)


def _solve_one(res, x0, tol=1e-13, maxiter=30):
    x, err = batched_newton(lambda X: np.stack([res(r) for r in X]), x0[None, :], tol, maxiter)
    if err[0] >= 1e-9:
        raise RuntimeError("controller init residual %g exceeds 1e-9" % err[0])
    return x[0]
