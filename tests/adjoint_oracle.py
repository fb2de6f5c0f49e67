"""CPU restatement of the discrete adjoint (test infrastructure only).

The forward run is the oracle's integrate! restatement; the adjoint sweeps
its solves backwards with dense linear algebra on the oracle's BE Jacobian:
    J_s^T lambda_s = dJ/dy_s + E lambda_{s+1},   dJ/dp = -sum_s lambda_s^T dF_s/dp,
    dJ/dz0 = E lambda_1,
where s runs over every Newton solve (regular steps and the dt = 0 re-solves
after an event), E selects the differential rows, and dF_s/dp comes from
central differences of the oracle's residual.  The objective is
    J = sum_{t=1..n} dt * (w_speed * sum_gen w^2 + w_volt * sum_bus max(0, v_min - |V|)^2),
the time weighting of the reference's objective (src/nlp.jl:30-46,
examples/adjoint.jl:75-82) applied to its functional (src/dynamics.jl:330-337);
the event offsets follow test/test_adjoint_event_offset.jl:1-25 (the
Jacobian of the solve that produced traj[:, i] is taken with the fault
status of that solve).

The reference's own adjoint is no longer in its sources (src/nlp.jl:50-53),
so this is pinned against central finite differences of the oracle's
integration (the check examples/adjoint.jl and the event-offset test make).
"""
import numpy as np

from helpers import LY


def objective_terms(PA, y, w_speed, w_volt, v_min):
    """r(y) and dr/dy for one state vector."""
    n_bus = PA.n_bus
    net = PA.n_diff + PA.n_alg
    g = np.zeros_like(y)
    wi = PA.tables[0].diff_ptr + 4
    w = y[wi]
    r = w_speed * np.sum(w * w)
    g[wi] += w_speed * 2.0 * w
    if w_volt != 0.0:
        vr_i = net + 2 * np.arange(n_bus)
        vr, vi = y[vr_i], y[vr_i + 1]
        vm = np.hypot(vr, vi)
        s = v_min - vm
        on = (s > 0) & (vm > 0)
        r += w_volt * np.sum(np.where(on, s * s, 0.0))
        k = np.where(on, -w_volt * 2.0 * s / np.where(vm > 0, vm, 1.0), 0.0)
        g[vr_i] += k * vr
        g[vr_i + 1] += k * vi
    return r, g


def objective_of_traj(PA, traj, dt, w_speed=1.0, w_volt=0.0, v_min=0.9):
    """J for trajectories [M, n+1, n_sys] (points 1..n)."""
    out = np.zeros(traj.shape[0])
    for m in range(traj.shape[0]):
        for t in range(1, traj.shape[1]):
            out[m] += dt * objective_terms(PA, traj[m, t], w_speed, w_volt, v_min)[0]
    return out


def fault_status(on_steps, off_steps, upto):
    a, b = np.asarray(on_steps), np.asarray(off_steps)
    return ((a <= upto) & ~((b <= upto) & (b >= a))).astype(np.uint8)


def newton_dense(orc, PA, y0, zold, u, p, fa, nf, on, dt, tol=1e-13, itermax=50):
    y = y0.copy()
    for _ in range(itermax):
        f = orc.residual(PA, y, zold, u, p, fa, nf, on, dt)
        if np.max(np.abs(f)) < tol:
            break
        y -= np.linalg.solve(orc.jacobian_dense(PA, y, u, p, fa, nf, on, dt), f)
    return y


def adjoint(orc, PA, z0, u, p, events, dt, nsteps, w_speed=1.0, w_volt=0.0, v_min=0.9, tol=1e-12, params=None):
    """J, dJ/dp [n_par], dJ/dz0 [n_sys] for one scenario whose faults are
    `events` (a list of model.ContingencyEvent); dJ/dp only for the indices
    `params` (default: all)."""
    cols = list(range(p.size)) if params is None else list(params)
    fa, nf = LY.fault_array([events], dt)
    ons = [fa[e].on_step for e in range(nf)]
    offs = [fa[e].off_step for e in range(nf)]
    ev_steps = set(ons) | set(offs)
    r = orc.integrate(PA, z0[None, :], u[None, :], p[None, :], fa, nf, dt, nsteps, tol=tol, itermax=50)
    traj = r["traj"][0]
    # the dt = 0 re-solves: from the state after step k with the new status
    resolved = {}
    for k in sorted(ev_steps):
        if 1 <= k <= nsteps:
            on = fault_status(ons, offs, k)
            resolved[k] = newton_dense(orc, PA, traj[k], traj[k], u, p, fa, nf, on, 0.0)
    diff = np.asarray(PA.is_diff, dtype=bool)
    E = np.concatenate([diff, np.zeros(PA.n_sys - diff.size, dtype=bool)])

    def dFdp(y, zold, on, dts):
        out = np.zeros((PA.n_sys, p.size))
        for j in cols:
            h = 1e-6 * max(1.0, abs(p[j]))
            pp, pm = p.copy(), p.copy()
            pp[j] += h
            pm[j] -= h
            out[:, j] = (orc.residual(PA, y, zold, u, pp, fa, nf, on, dts) -
                         orc.residual(PA, y, zold, u, pm, fa, nf, on, dts)) / (2 * h)
        return out

    g = np.zeros(PA.n_sys)
    grad = np.zeros(p.size)
    J = 0.0
    for k in range(nsteps, 0, -1):
        if k in resolved:
            on = fault_status(ons, offs, k)
            y = resolved[k]
            Jm = orc.jacobian_dense(PA, y, u, p, fa, nf, on, 0.0)
            lam = np.linalg.solve(Jm.T, g)
            grad -= lam @ dFdp(y, traj[k], on, 0.0)
            g = np.where(E, lam, 0.0)
        on = fault_status(ons, offs, k - 1)
        y = traj[k]
        rv, rg = objective_terms(PA, y, w_speed, w_volt, v_min)
        J += dt * rv
        g = g + dt * rg
        zold = resolved.get(k - 1, traj[k - 1])
        Jm = orc.jacobian_dense(PA, y, u, p, fa, nf, on, dt)
        lam = np.linalg.solve(Jm.T, g)
        grad -= lam @ dFdp(y, zold, on, dt)
        g = np.where(E, lam, 0.0)
    return J, grad, g


def fd_gradient(orc, PA, z0, u, p, events, dt, nsteps, idx, w_speed=1.0, w_volt=0.0, v_min=0.9, rel=1e-5,
                tol=1e-12, nthreads=8):
    """Central differences of J with respect to p[idx], one oracle run of
    2 * len(idx) perturbed scenarios."""
    idx = list(idx)
    Mf = 2 * len(idx)
    P = np.tile(p, (Mf, 1))
    hs = []
    for q, j in enumerate(idx):
        h = rel * max(1.0, abs(p[j]))
        hs.append(h)
        P[2 * q, j] += h
        P[2 * q + 1, j] -= h
    fa, nf = LY.fault_array([events] * Mf, dt)
    r = orc.integrate(PA, np.tile(z0, (Mf, 1)), np.tile(u, (Mf, 1)), P, fa, nf, dt, nsteps, tol=tol, itermax=50,
                      nthreads=nthreads)
    Jv = objective_of_traj(PA, r["traj"], dt, w_speed, w_volt, v_min)
    return np.array([(Jv[2 * q] - Jv[2 * q + 1]) / (2 * hs[q]) for q in range(len(idx))])


def differentiated_params(PA):
    """Parameter indices the GPU adjoint differentiates: machine H and D,
    SEXS K, ESDC1A KA, TGOV1 R, IEESGO K1."""
    T = PA.tables
    idx = list(T[0].par_ptr + 6) + list(T[0].par_ptr + 7)
    idx += list(T[1].par_ptr + 6) + list(T[2].par_ptr) + list(T[3].par_ptr + 2) + list(T[4].par_ptr)
    return sorted(int(i) for i in idx)
