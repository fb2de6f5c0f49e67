"""CPU tests of the host side: setup, descriptor export, the C-ABI library's
symbols and its host-only symbolic analysis, and scenario sharding across
ranks (gloo)."""
import ctypes as C
import os
import re

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from conftest import ROOT
from helpers import LY, Case, M, psse, psse_case, synthetic

HEADER = os.path.join(ROOT, "include", "gradpower_gb300.h")


@pytest.fixture(scope="module")
def lib():
    import subprocess
    import shutil
    if shutil.which(os.environ.get("NVCC", "nvcc")) is None:
        pytest.skip("nvcc not available")
    from gradpower_gb300 import build, gpu
    build.build()
    return gpu.library()


def test_library_exports_every_declared_symbol(lib):
    names = re.findall(r"^\w[\w\s\*]*?\b(gp_\w+)\(", open(HEADER).read(), re.M)
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert lib.gp_abi_version() == 1


def test_recip_check_validates_its_arguments_before_any_device_call(lib):
    """gp_recip_check refuses a negative count or missing arrays, and an
    empty call succeeds, all without touching a device."""
    assert lib.gp_recip_check(-1, None, None) == -1
    assert "bad arguments" in lib_error(lib)
    assert lib.gp_recip_check(3, None, None) == -1
    assert lib.gp_recip_check(0, None, None) == 0


def lib_error(lib):
    buf = C.create_string_buffer(1024)
    lib.gp_last_error(buf, 1024)
    return buf.value.decode(errors="replace")


def _reduced_S(ps, rng):
    """A reduced matrix with the structure the library expects: -Ybus off the
    diagonal blocks, random well-conditioned diagonal blocks."""
    Y = ps.ybus.tocoo()
    nb = ps.nbus
    r, c, v = [], [], []
    for i, j, y in zip(Y.row, Y.col, Y.data):
        r += [2 * i, 2 * i, 2 * i + 1, 2 * i + 1]
        c += [2 * j, 2 * j + 1, 2 * j, 2 * j + 1]
        v += [-y.real, y.imag, -y.imag, -y.real]
    for i in range(nb):
        for a in range(2):
            for b in range(2):
                r.append(2 * i + a)
                c.append(2 * i + b)
                v.append(0.5 * rng.normal() + (3.0 if a == b else 0.0))
    S = sp.csr_matrix((v, (r, c)), shape=(2 * nb, 2 * nb))
    S.sum_duplicates()
    S.sort_indices()
    return S


@pytest.mark.parametrize("name", ["two_bus", "ring39", "planar2k", "planar70k"])
def test_reduced_factorisation_matches_scipy(lib, name):
    """Symbolic analysis + front assembly + multifrontal LU/solves (host
    emulation of the device kernels) against scipy's sparse LU."""
    w = synthetic.WORKLOADS[name]()
    PA = LY.ProblemArrays(w.ps)
    P = PA.as_ctypes()
    rng = np.random.default_rng(0)
    S = _reduced_S(w.ps, rng)
    rhs = rng.normal(size=S.shape[0])
    x = np.zeros_like(rhs)
    out = np.zeros(12)
    rp, ci, sv = S.indptr.astype(np.int32), S.indices.astype(np.int32), S.data.astype(np.float64)
    lib.gp_reduced_selftest.argtypes = [C.c_void_p] * 7
    rc = lib.gp_reduced_selftest(C.addressof(P), rp.ctypes.data, ci.ctypes.data, sv.ctypes.data,
                                 rhs.ctypes.data, x.ctypes.data, out.ctypes.data)
    assert rc == 0, lib_error(lib)
    assert out[0] == 0.0 and out[1] == 0
    # blocked triangular solves (staging indices checked) agree with the
    # level-order solves
    assert out[4] <= 1e-13 and out[5] >= 1
    # S^T from the transposed assembly lists (the adjoint's system)
    assert out[8] <= 1e-10
    # the split-front elimination (parts emulated) gives the same bits
    assert out[11] == 0.0
    xr = spla.spsolve(S.tocsc(), rhs)
    assert np.max(np.abs(x - xr)) <= 1e-12 * np.max(np.abs(xr))


def test_reduced_factorisation_with_static_generators(lib, golden_cases, orc):
    """IEEE 9-bus with the slack machine (bus 1) and one PV machine (bus 2)
    left without a dynamic model: StaticGenerator stand-ins add algebraic
    states to the reduced system (PV: q; slack: p, q)."""
    ps, dp = psse_case(golden_cases, "ieee9_v33.raw", "ieee9bus_gov.dyr", drop_dyr_gens=(1, 2))
    PA = LY.ProblemArrays(ps)
    kinds = [ps.dynamic.devices[i].dtype.bus_type for i in PA.tables[7].device_index]
    assert sorted(kinds) == [2, 3]
    # true reduced matrix from the oracle's Jacobian at a perturbed state
    fa, nf = LY.fault_array([[]], 1 / 120)
    z = dp.zvec + 1e-3 * np.random.default_rng(1).normal(size=dp.zvec.size)
    J = orc.jacobian_dense(PA, z, dp.uvec, dp.pvec, fa, nf, np.zeros(1, np.uint8), 1 / 120)
    net = PA.n_diff + PA.n_alg
    red = [i for i in range(PA.n_sys) if i >= net]
    sg_states = []
    for k, i in enumerate(PA.tables[7].device_index):
        rec = ps.dynamic.devices[i]
        sg_states += list(range(rec.alg_ptr, rec.alg_ptr + rec.dtype.alg_size))
    red_global = [net + j for j in range(2 * PA.n_bus)] + sg_states
    w_idx = [i for i in range(net) if i not in set(sg_states)]
    A = J[np.ix_(w_idx, w_idx)]
    S = J[np.ix_(red_global, red_global)] - J[np.ix_(red_global, w_idx)] @ np.linalg.solve(A, J[np.ix_(w_idx, red_global)])
    Ssp = sp.csr_matrix(np.where(np.abs(S) > 0, S, 0.0))
    # keep the structural entries of the static generator coupling
    Ssp.sort_indices()
    rhs = np.random.default_rng(2).normal(size=len(red_global))
    x = np.zeros_like(rhs)
    out = np.zeros(12)
    P = PA.as_ctypes()
    rp, ci, sv = Ssp.indptr.astype(np.int32), Ssp.indices.astype(np.int32), Ssp.data.astype(np.float64)
    lib.gp_reduced_selftest.argtypes = [C.c_void_p] * 7
    assert lib.gp_reduced_selftest(C.addressof(P), rp.ctypes.data, ci.ctypes.data, sv.ctypes.data,
                                   rhs.ctypes.data, x.ctypes.data, out.ctypes.data) == 0
    assert out[0] < 1e-12
    # S^T, whose static-generator couplings are not symmetric
    assert out[8] <= 1e-10
    xr = np.linalg.solve(S, rhs)
    assert np.max(np.abs(x - xr)) <= 1e-10 * np.max(np.abs(xr))


def test_synthetic_sizes():
    """Sizes of the benchmark grids (ring39: 228 unknowns, 461 parameters;
    planar2k: cluster widths 15..27)."""
    w = synthetic.ring39()
    assert len(w.dp.zvec) == 228 and w.ps.dynamic.par_dim == 461 and len(w.faults) == 64
    w2 = synthetic.planar2k()
    widths = {c.w_size for c in w2.ps.dynamic.clusters}
    assert widths == {15, 16, 18, 19, 23, 24, 26, 27}
    assert len(w2.ps.branches) == 2700 and w2.n_scenarios == 256


def test_julia_round_ties_to_even():
    assert LY.jl_round(2.5) == 2 and LY.jl_round(3.5) == 4 and LY.jl_round(0.1 / (1 / 120)) == 12


def test_fault_array_expansion():
    evs = [[M.ContingencyEvent(1, 0.1, 0.1, 0.2)], [], [M.ContingencyEvent(0, 0.2, 0.05, 0.3)]]
    arr, n = LY.fault_array(evs, 1 / 120, [M.ContingencyEvent(2, 0.5, 0.5, 0.6)])
    rows = [(arr[k].scenario, arr[k].bus, arr[k].on_step, arr[k].off_step) for k in range(n)]
    assert rows == [(-1, 2, 60, 72), (0, 1, 12, 24), (2, 0, 6, 36)]


def test_psse_reader(golden_cases):
    ps = psse.ps_from_records(golden_cases["raw"]["ieee9_v33.raw"])
    assert ps.nbus == 9 and len(ps.gens) == 3 and len(ps.loads) == 3
    assert len(ps.branches) == 9          # 6 lines + 3 transformers
    assert ps.loads[0].qd < 0             # stored negated (src/parse.jl:384)
    assert ps.buses[0].type == M.SLACK and ps.buses[0].v0m == 1.04


def test_cluster_layout_matches_reference_order(golden_cases):
    """Cluster-contiguous z: generator diff, generator alg, governor diff,
    governor alg, ... then (vr, vi) per bus (src/clusters.jl:218-223)."""
    ps, dp = psse_case(golden_cases, "ieee9_v33.raw", "ieee9bus_gov.dyr")
    d = ps.dynamic
    cl = d.clusters[0]
    g, gv = d.devices[cl.gen], d.devices[cl.gov]
    assert g.diff_ptr == cl.w_start and g.alg_ptr == cl.w_start + 6
    assert gv.diff_ptr == cl.w_start + 10 and gv.alg_ptr == cl.w_start + 15
    assert d.uvec_idx[g.ctrl_ptr + 1] == gv.alg_ptr       # p_m <- governor output
    assert d.uvec_idx[gv.ctrl_ptr] == g.diff_ptr + 4      # governor reads w


def _gloo_worker(rank, world, port, out_q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from conftest import load_oracle, load_package
    gp = load_package()
    orc = load_oracle()
    from gradpower_gb300 import gpu as G
    w = gp.synthetic.ring39()
    Mtot = 6
    lo, hi = G.scenario_shard(Mtot, rank, world)
    c = Case(w.ps, w.dp, w.faults[lo:hi], hi - lo)
    z, u, p = c.arrays()
    fa, nf = c.fault_array()
    r = orc.integrate(c.PA, z, u, p, fa, nf, 1 / 120, 30, itermax=30)
    parts = [None] * world
    dist.all_gather_object(parts, (lo, hi, r["z"], r["iters"]))
    if rank == 0:
        out_q.put(parts)
    dist.destroy_process_group()


def test_scenario_shard_partitions_the_scenarios():
    """The ranks' ranges are contiguous, cover every scenario once, and
    differ in size by at most one (more ranks than scenarios included)."""
    from gradpower_gb300 import gpu as G
    for Mtot in range(0, 21):
        for world in range(1, 10):
            r = [G.scenario_shard(Mtot, k, world) for k in range(world)]
            assert r[0][0] == 0 and r[-1][1] == Mtot
            assert all(r[k][1] == r[k + 1][0] for k in range(world - 1))
            sizes = [hi - lo for lo, hi in r]
            assert min(sizes) >= 0 and max(sizes) - min(sizes) <= 1


def test_scenario_sharding_gloo(orc):
    """Scenarios shard across ranks with no exchange during the run; the
    gathered result equals the single-process run (world size 2, gloo)."""
    import multiprocessing as mp
    import random
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = random.randint(20000, 40000)
    procs = [ctx.Process(target=_gloo_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    parts = q.get(timeout=240)
    for pr in procs:
        pr.join(timeout=60)
    w = synthetic.ring39()
    c = Case(w.ps, w.dp, w.faults[:6], 6)
    z, u, p = c.arrays()
    fa, nf = c.fault_array()
    full = orc.integrate(c.PA, z, u, p, fa, nf, 1 / 120, 30, itermax=30)
    for lo, hi, zf, it in parts:
        assert np.array_equal(zf, full["z"][lo:hi])
        assert np.array_equal(it, full["iters"][lo:hi])


CLUSTER_CASES = [("2bus.raw", "2bus_ESDC1A.dyr"), ("2bus.raw", "2bus_SEXS.dyr"), ("2bus.raw", "2bus_TGOV1.dyr"),
                 ("2bus.raw", "2bus_IEESGO.dyr"), ("ieee9_v33.raw", "ieee9bus_gov.dyr"),
                 ("IEEE39.raw", "IEEE39_gov.dyr"), ("IEEE39.raw", "IEEE39.dyr"), "ring39"]


@pytest.mark.parametrize("case", CLUSTER_CASES, ids=lambda c: c if isinstance(c, str) else c[1])
def test_cluster_factorisation_matches_dense_solves(lib, golden_cases, orc, case):
    """Static-pivot sparse LU of every generator cluster (host run of the
    device program) against dense solves with the oracle's Jacobian blocks:
    A_k^-1 f_k, A_k^-1 B_k, C_k A_k^-1 B_k and C_k A_k^-1 f_k."""
    if isinstance(case, str):
        w = synthetic.WORKLOADS[case]()
        ps, dp = w.ps, w.dp
    else:
        ps, dp = psse_case(golden_cases, *case)
    PA = LY.ProblemArrays(ps)
    P = PA.as_ctypes()
    dt = 1 / 120
    rng = np.random.default_rng(7)
    zold = dp.zvec.copy()
    z = zold + 1e-3 * rng.normal(size=zold.size)
    fa, nf = LY.fault_array([[]], dt)
    J = orc.jacobian_dense(PA, z, dp.uvec, dp.pvec, fa, nf, np.zeros(1, np.uint8), dt)
    f = orc.residual(PA, z, zold, dp.uvec, dp.pvec, fa, nf, np.zeros(1, np.uint8), dt)
    net = PA.n_diff + PA.n_alg
    yx = np.zeros(3 * net)
    nt = int((PA.cl_gen >= 0).sum())
    clout = np.zeros((max(nt, 1), 8))
    fc = np.zeros(net)
    out = np.zeros(4)
    assert lib.gp_cluster_selftest(C.addressof(P), z.ctypes.data, zold.ctypes.data, dp.uvec.ctypes.data,
                                   dp.pvec.ctypes.data, dt, yx.ctypes.data, clout.ctypes.data,
                                   fc.ctypes.data, out.ctypes.data) == 0
    assert out[1] >= 1 and out[2] > 0
    fmax = 0.0
    k = 0
    for c in range(PA.n_clusters):
        if PA.cl_gen[c] < 0:
            continue
        w0, W, b = PA.cl_w_start[c], PA.cl_w_size[c], PA.cl_bus[c]
        s = slice(w0, w0 + W)
        rows = [net + 2 * b, net + 2 * b + 1]
        A = J[s, s]
        B = J[s][:, rows]
        Cm = J[rows][:, s]
        # the device equations take each division by a parameter once, as a
        # reciprocal: the same residual to rounding (terms up to ~1/x''_d)
        assert np.max(np.abs(fc[s] - f[s])) <= 1e-12 * max(1.0, np.max(np.abs(f[s])))
        fmax = max(fmax, np.max(np.abs(f[s])))
        y = np.linalg.solve(A, f[s])
        X = np.linalg.solve(A, B)
        got = np.stack([yx[s], yx[net:][s], yx[2 * net:][s]], axis=1)
        ref = np.concatenate([y[:, None], X], axis=1)
        assert np.max(np.abs(got - ref)) <= 1e-11 * max(1.0, np.max(np.abs(ref))), c
        CX = Cm @ X
        Cy = Cm @ y
        assert np.allclose(clout[k, :4], CX.ravel(), rtol=1e-11, atol=1e-12), c
        assert np.allclose(clout[k, 4:6], Cy, rtol=1e-11, atol=1e-13), c
        k += 1
    assert k == nt
    assert abs(out[0] - fmax) <= 1e-15 * max(1.0, fmax)


def test_generator_outputs_match_apply_pf_solution():
    """gpu.generator_outputs (the power-flow write-back vectorised over
    scenarios) equals model.apply_pf_solution run on each scenario's scaled
    copy of the system."""
    import copy
    from gradpower_gb300 import gpu
    w = synthetic.planar2k()
    ps = w.ps
    rng = np.random.default_rng(5)
    scales = np.array([0.95, 1.0, 1.04])
    vm = np.array([[b.v0m for b in ps.buses]] * 3) * (1.0 + 1e-3 * rng.standard_normal((3, ps.nbus)))
    va = np.array([[b.v0a for b in ps.buses]] * 3) + 1e-3 * rng.standard_normal((3, ps.nbus))
    psch, qsch = gpu.generator_outputs(ps, vm, va, scales, scales)
    slack = {i for i, b in enumerate(ps.buses) if b.type == M.SLACK}
    assert any(ps.buses[g.bus].type == M.PV for g in ps.gens) and any(g.bus in slack for g in ps.gens)
    for m, s in enumerate(scales):
        ps2 = copy.deepcopy(ps)
        for l in ps2.loads:
            l.pd *= s
            l.qd *= s
        for g in ps2.gens:
            if g.bus not in slack:
                g.psch *= s
        M.apply_pf_solution(ps2, vm[m], va[m])
        assert np.allclose(psch[m], [g.psch for g in ps2.gens], rtol=0, atol=1e-12)
        assert np.allclose(qsch[m], [g.qsch for g in ps2.gens], rtol=0, atol=1e-12)


def test_disconnect_array_names_table_rows():
    """layout.disconnect_array finds each device's table and row as
    _set_device_offline! does (its rank among the devices of its type),
    expands per-scenario and global events, and rounds steps like the
    reference's schedule."""
    w = synthetic.ring39()
    PA = LY.ProblemArrays(w.ps)
    ZL, SX = PA.tables[LY.GP_ZIPLOAD], PA.tables[LY.GP_SEXS]
    dz, dx = int(ZL.device_index[3]), int(SX.device_index[1])
    arr, n = LY.disconnect_array(PA, [[M.DisconnectDeviceEvent(dz, 0.05)], [], [M.DisconnectDeviceEvent(dx, 0.1)]],
                                 1.0 / 120.0, [M.DisconnectDeviceEvent(dx, 0.2)])
    rows = [(arr[k].scenario, arr[k].type, arr[k].index, arr[k].on_step) for k in range(n)]
    assert rows == [(-1, LY.GP_SEXS, 1, 24), (0, LY.GP_ZIPLOAD, 3, 6), (2, LY.GP_SEXS, 1, 12)]
    with pytest.raises(ValueError):
        LY.disconnect_array(PA, [[M.DisconnectDeviceEvent(10 ** 6, 0.05)]], 1.0 / 120.0)
