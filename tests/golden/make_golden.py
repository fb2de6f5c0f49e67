"""Generate the golden fixtures of this directory from the reference tree.

Run where the reference is checked out, with its root given as the first
argument or in GRADPOWER_REFERENCE.  Outputs, all JSON:

  cases.json      the reference's example cases (examples/2bus*.raw|dyr,
                  ieee9_v33.raw + ieee9bus*.dyr, IEEE39.raw + IEEE39*.dyr,
                  test/testdata/2bus.*), tokenised by psse.read_raw / read_dyr
  known.json      known-answer values stated in the reference's tests:
                  - MATPOWER case 9 system and voltages (test/test_case9data.jl,
                    test/test_pflow.jl:11-26)
                  - 2-bus final-state values (test/test_dynamics.jl:25-28)
                  - the uqgrid 2-bus GENROU+ESDC1A rotor-speed trajectory
                    (examples/refs/2bus_esdc1a.npz, every 5th sample)

The numbers are read from the reference files; nothing is typed in by hand.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GRADPOWER_REFERENCE", "")
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _load_psse():
    import importlib.util
    root = os.path.dirname(os.path.dirname(HERE))
    pkg = os.path.join(root, "gradpower.jl_gb300")
    spec = importlib.util.spec_from_file_location("gradpower_gb300", os.path.join(pkg, "__init__.py"),
                                                  submodule_search_locations=[pkg])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gradpower_gb300"] = mod
    spec.loader.exec_module(mod)
    from gradpower_gb300 import psse
    return psse


def cases(psse):
    ex = os.path.join(REF, "examples")
    out = {"raw": {}, "dyr": {}}
    for f in sorted(os.listdir(ex)):
        path = os.path.join(ex, f)
        if f.endswith(".raw"):
            out["raw"][f] = psse.read_raw(open(path).read())
        elif f.endswith(".dyr"):
            out["dyr"][f] = psse.read_dyr(open(path).read())
    td = os.path.join(REF, "test", "testdata")
    out["raw"]["testdata/2bus.raw"] = psse.read_raw(open(os.path.join(td, "2bus.raw")).read())
    out["dyr"]["testdata/2bus.dyr"] = psse.read_dyr(open(os.path.join(td, "2bus.dyr")).read())
    return out


def _julia_calls(text, name):
    return [m.group(1) for m in re.finditer(r"push!\(\w+, %s\((.*?)\)\)" % name, text)]


def _args(s):
    return [a.strip().strip('"') for a in s.split(",")]


def known():
    t = open(os.path.join(REF, "test", "test_case9data.jl")).read()
    case9 = {
        "baseMVA": float(re.search(r"baseMVA = ([0-9.]+)", t).group(1)),
        "buses": [_args(a) for a in _julia_calls(t, "Bus")],
        "gens": [_args(a) for a in _julia_calls(t, "Gen")],
        "loads": [_args(a) for a in _julia_calls(t, "Load")],
        "branches": [_args(a) for a in _julia_calls(t, "Branch")],
    }
    pf = open(os.path.join(REF, "test", "test_pflow.jl")).read()
    body = pf[pf.index("vmat = ["):pf.index("]", pf.index("vmat = ["))]
    vm = []
    for re_, sign, im_ in re.findall(r"([-0-9.]+) ([+-]) ([0-9.]+)im", body):
        vm.append([float(re_), float(im_) * (1 if sign == "+" else -1)])
    dyn = open(os.path.join(REF, "test", "test_dynamics.jl")).read()
    vals = {int(i): float(v) for i, v in re.findall(r"isapprox\(result\[(\d+)\], ([-0-9.eE]+), rtol=1e-2\)", dyn)}
    ev = re.search(r"ContingencyEvent\((\d+), ([0-9.]+), ([0-9.]+), ([0-9.]+)\)", dyn)
    d = np.load(os.path.join(REF, "examples", "refs", "2bus_esdc1a.npz"))
    hist = d["history"]
    sidx = int(np.asarray(d["speed_idx"]).ravel()[0])
    step = 5
    uq = {
        "tvec": d["tvec"][::step].tolist(),
        "speed": hist[sidx, ::step].tolist(),
        "speed_idx": sidx,
        "fault_bus_index": int(d["fault_bus"]),
        "rfault": float(d["rfault"]), "ton": float(d["ton"]), "toff": float(d["toff"]),
        "dt": float(d["dt"]), "tend": float(d["tend"]), "zipload_alpha": float(d["zipload_alpha"]),
    }
    return {
        "case9": case9,
        "case9_vmatpower": vm,
        "dynamics_2bus": {"values_1based": vals,
                          "event": [int(ev.group(1)), float(ev.group(2)), float(ev.group(3)), float(ev.group(4))],
                          "tfinal": 1.0, "rtol": 1e-2},
        "uqgrid_2bus_esdc1a": uq,
    }


if __name__ == "__main__":
    if not REF or not os.path.isdir(REF):
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set GRADPOWER_REFERENCE)")
    psse = _load_psse()
    with open(os.path.join(HERE, "cases.json"), "w") as f:
        json.dump(cases(psse), f)
    with open(os.path.join(HERE, "known.json"), "w") as f:
        json.dump(known(), f, indent=1)
    print("wrote", os.listdir(HERE))
