"""Minimal PSS/E v33 .raw / .dyr reader.

Restates the parts of the reference's case import that this path needs:
`read_psse_raw` (src/parse_psse_raw.jl) for bus, load, fixed-shunt,
generator, branch and two-winding transformer records; `raw_to_grad`
(src/parse.jl:212-400) with its conventions (load Q stored negated, PV/slack
voltage set point taken from the generator, PV buses without an active
generator demoted to PQ, transformer impedance on the system base);
`read_psse_dyr` (src/parse.jl:130-170) and `create_device_vector`
(src/parse.jl:405-480) with its three-pass filter (machines matched to an
active static generator, then controllers whose machine survived, then
stabilisers whose exciter survived); and `from_psse` (src/parse.jl:81-103).

Records can be read from files (`read_raw`, `read_dyr`) or passed in already
tokenised (`ps_from_records`, `devices_from_records`), which is how the
golden fixtures under tests/golden carry the reference's example cases.
"""
from __future__ import annotations

import math
import re
from typing import Dict, List, Optional

from . import model as M

_SECTIONS = ["bus", "load", "fixed_shunt", "generator", "branch", "transformer"]


def _split_record(line: str) -> List[str]:
    line = line.split("/")[0]
    return [t.strip() for t in re.split(r",", line) if t.strip() != ""] if "," in line else line.split()


def read_raw(text: str) -> Dict[str, list]:
    """Tokenise the sections of a v33 .raw file this path uses."""
    lines = text.splitlines()
    head = _split_record(lines[0])
    rec: Dict[str, list] = {"baseMVA": float(head[1])}
    i = 3
    for sec in _SECTIONS:
        rec[sec] = []
        while i < len(lines):
            ln = lines[i]
            if ln.strip().startswith("0 ") or ln.strip() == "0" or ln.strip().startswith("0/"):
                i += 1
                break
            if sec == "transformer":
                t1 = _split_record(lines[i])
                k = int(t1[2])
                n = 4 if k == 0 else 5
                rec[sec].append([_split_record(lines[i + j]) for j in range(n)])
                i += n
            else:
                rec[sec].append(_split_record(ln))
                i += 1
    return rec


def read_dyr(text: str) -> List[List[str]]:
    """Dynamic records as token lists; a record ends at a line whose last
    token is '/' (src/parse.jl:141-170)."""
    out = []
    cur: Optional[List[str]] = None
    for ln in text.splitlines():
        s = ln.strip()
        if cur is None:
            if not s or s.startswith("//"):
                continue
            cur = [t for t in (re.split(r"\s*,\s*", s) if "," in s else re.split(r"\s+", s))]
        else:
            cur.extend(t for t in re.split(r"\s*,\s*|\s+", s))
        if cur and cur[-1] == "/":
            out.append(cur)
            cur = None
    return out


def _q(s: str) -> str:
    return s.strip().strip("'").strip()


def ps_from_records(rec: Dict[str, list]) -> M.PowerSystem:
    """`raw_to_grad` restated (src/parse.jl:212-400)."""
    base = rec["baseMVA"]
    buses, busmap = [], {}
    for k, r in enumerate(rec["bus"]):
        busmap[int(r[0])] = k
        buses.append(M.Bus(int(r[0]), _q(r[1]), int(r[3]), float(r[2]), float(r[7]),
                           math.pi / 180.0 * float(r[8])))
    branches = []
    for r in rec["branch"]:
        if int(r[13]) != 1:
            continue
        branches.append(M.Branch(busmap[int(r[0])], busmap[int(r[1])], _q(r[2]), float(r[3]),
                                 float(r[4]), float(r[5]), 0.0, 0.0))
    shunts = []
    for t in rec["transformer"]:
        l1, l2, l3, l4 = t[0], t[1], t[2], t[3]
        if int(l1[11]) != 1:
            continue
        fr, to = busmap[int(l1[0])], busmap[int(l1[1])]
        CW, CZ = int(l1[4]), int(l1[5])
        if CW == 2:
            raise ValueError("transformer winding code CW=2 is not supported (as in the reference)")
        v1, v2 = float(l3[0]), float(l4[0])
        nomv1 = float(l3[1])
        zr = (nomv1 / buses[fr].baseKV) ** 2.0 if (CW == 1 and nomv1 > 0.0) else 1.0
        r_, x_ = float(l2[0]), float(l2[1])
        if CZ == 1:
            r12, x12 = r_ * v2 ** 2.0 * zr, x_ * v2 ** 2.0 * zr
        elif CZ == 2:
            sb = float(l2[2])
            r12, x12 = r_ * (base / sb) * v2 ** 2.0, x_ * (base / sb) * v2 ** 2.0
        else:
            raise ValueError("transformer CZ=3 is not supported (as in the reference)")
        mag1, mag2 = float(l1[7]), float(l1[8])
        mag_sh = mag2 if abs(mag2) > 0.0 else 0.0
        branches.append(M.Branch(fr, to, _q(l1[3]), r12, x12, mag_sh, v1 / v2, float(l3[2])))
        if int(l3[6]) == 1:
            shunts.append(M.Shunt(fr, "tran", mag1 * base, mag2 * base))
    with_gen = set()
    for r in rec["generator"]:
        if int(r[14]) == 1:
            with_gen.add(busmap[int(r[0])])
    gens = []
    for r in rec["generator"]:
        if int(r[14]) != 1:
            continue
        b = busmap[int(r[0])]
        gens.append(M.Gen(b, _q(r[1]), float(r[2]) / base, float(r[3]) / base, float(r[8])))
        if buses[b].type in (M.PV, M.SLACK):
            buses[b].v0m = float(r[6])
    for k, bus in enumerate(buses):
        if bus.type == M.PV and k not in with_gen:
            bus.type = M.PQ
    loads = []
    for r in rec["load"]:
        if int(r[2]) != 1:
            continue
        loads.append(M.Load(busmap[int(r[0])], _q(r[1]), float(r[5]) / base, -float(r[6]) / base))
    for r in rec["fixed_shunt"]:
        if int(r[2]) != 1:
            continue
        shunts.append(M.Shunt(busmap[int(r[0])], _q(r[1]), float(r[3]) / base, float(r[4]) / base))
    return M.PowerSystem(base, buses, gens, loads, branches, shunts, busmap)


def _f(tok: List[str], i: int) -> float:
    return float(tok[i - 1])


def _device(tok: List[str]) -> Optional[M.Device]:
    kind = tok[1].strip("'").strip()
    bus = int(tok[0])
    ident = tok[2]
    n = len(tok)
    if kind == "GENROU":
        S1 = _f(tok, 16) if n >= 17 else 0.0
        S2 = _f(tok, 17) if n >= 18 else 0.0
        return M.Genrou(bus, ident, _f(tok, 10), _f(tok, 11), _f(tok, 12), _f(tok, 13), _f(tok, 14),
                        _f(tok, 15), _f(tok, 8), _f(tok, 9), _f(tok, 4), _f(tok, 6), _f(tok, 5),
                        _f(tok, 7), S1, S2)
    if kind == "GENSAL":
        S1 = _f(tok, 14) if n >= 15 else 0.0
        S2 = _f(tok, 15) if n >= 16 else 0.0
        return M.Genrou.gensal(bus, ident, _f(tok, 9), _f(tok, 10), _f(tok, 11), _f(tok, 12),
                               _f(tok, 13), _f(tok, 7), _f(tok, 8), _f(tok, 4), _f(tok, 5),
                               _f(tok, 6), S1, S2)
    if kind == "IEESGO":
        return M.IEESGO(bus, ident, *[_f(tok, i) for i in range(4, 15)])
    if kind == "TGOV1":
        return M.TGOV1(bus, ident, *[_f(tok, i) for i in range(4, 11)])
    if kind == "SEXS":
        return M.SEXS(bus, ident, *[_f(tok, i) for i in range(4, 10)])
    if kind == "ESDC1A":
        sa, sb = M.esdc1a_sat_coefficients(_f(tok, 16), _f(tok, 17), _f(tok, 18), _f(tok, 19))
        return M.ESDC1A(bus, ident, _f(tok, 5), _f(tok, 6), _f(tok, 13), _f(tok, 14), _f(tok, 11),
                        _f(tok, 12), _f(tok, 4), sa, sb)
    if kind == "IEEEST":
        return M.IEEEST(bus, ident, int(tok[3]), int(tok[4]), *[_f(tok, i) for i in range(6, 23)])
    return None


def devices_from_records(dyr: List[List[str]], ps: M.PowerSystem) -> List[M.Device]:
    """`create_device_vector` restated (src/parse.jl:405-480)."""
    active = {(ps.buses[g.bus].i, M.normalize_id(g.id)) for g in ps.gens}
    parsed = [d for d in (_device(t) for t in dyr) if d is not None]
    out, kept_gen, kept_exc = [], set(), set()
    for d in parsed:
        if d.is_generator:
            key = (d.bus, M.normalize_id(d.id))
            if key in active:
                kept_gen.add(key)
                out.append(d)
    for d in parsed:
        if d.is_generator:
            continue
        key = (d.bus, M.normalize_id(d.id))
        if d.is_governor or d.is_exciter or d.is_stabilizer:
            if key not in kept_gen:
                continue
            if d.is_stabilizer:
                continue
            if d.is_exciter:
                kept_exc.add(key)
        out.append(d)
    for d in parsed:
        if d.is_stabilizer:
            key = (d.bus, M.normalize_id(d.id))
            if key in kept_gen and key in kept_exc:
                out.append(d)
    return out


def from_records(raw: Dict[str, list], dyr: List[List[str]], load_alpha: float = 1.0,
                 runpf: bool = True) -> M.PowerSystem:
    """`from_psse` + `build_network!` + `runpf!` + `set_dynamics!`, the
    order the reference's tests use (test/test_integrate.jl:6-16)."""
    ps = ps_from_records(raw)
    devs = devices_from_records(dyr, ps)
    psd = M.PowerSystemDynamics(devs)
    M.set_dynamics(ps, psd, load_alpha=load_alpha)
    M.build_network(ps)
    if runpf:
        M.runpf_inplace(ps)
        # ZIP loads read the solved |V| at init; StaticGenerator set points too
        for rec in psd.devices:
            if rec.dtype.kind == "static_gen":
                b = ps.buses[rec.bus]
                rec.dtype.vset, rec.dtype.aset = b.v0m, b.v0a
    return ps
