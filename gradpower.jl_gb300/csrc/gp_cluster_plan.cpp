// Host-once plan of the sparse cluster factorisation (see gp_cluster_plan.h).
#include "gp_cluster_plan.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <set>
#include <stdexcept>
#include <string>

namespace gp {
namespace {

struct PatSink {
    int ws;
    std::set<int> *ent;
    void put(int r, int c, double) { ent->insert((r - ws) * 32 + (c - ws)); }
    void putv(int r, int k, double) { ent->insert((r - ws) * 32 + 29 + k); }
    void putf(int r, double) { ent->insert((r - ws) * 32 + 31); }
};

struct DenseSink {
    int ws;
    double *a;   // [32*32]
    void put(int r, int c, double v) { a[(r - ws) * 32 + (c - ws)] = v; }
    void putv(int r, int k, double v) { a[(r - ws) * 32 + 29 + k] = v; }
    void putf(int r, double v) { a[(r - ws) * 32 + 31] = v; }
};

struct SlotSink {
    int ws;
    const short *slot_of;
    double *v;
    void put(int r, int c, double x) { v[slot_of[(r - ws) * 32 + (c - ws)]] = x; }
    void putv(int r, int k, double x) { v[slot_of[(r - ws) * 32 + 29 + k]] = x; }
    void putf(int r, double x) { v[slot_of[(r - ws) * 32 + 31]] = x; }
};

DevRef ref(const gp_device_table &T, int k) {
    DevRef d;
    d.dp = T.diff_ptr ? T.diff_ptr[k] : -1;
    d.ap = T.alg_ptr ? T.alg_ptr[k] : -1;
    d.cp = T.ctrl_ptr ? T.ctrl_ptr[k] : -1;
    d.pp = T.par_ptr[k];
    d.bus = T.bus[k];
    d.link0 = T.link0 ? T.link0[k] : -1;
    d.link1 = T.link1 ? T.link1[k] : -1;
    return d;
}

template <class Sink>
void eval_cluster(const gp_problem *pr, int c, const double *z, const double *u0, const double *p, Sink &s,
                  double *C, double *I) {
    const int net = pr->n_diff + pr->n_alg;
    genrou_eval(ref(pr->dev[GP_GENROU], pr->cl_gen[c]), net, z, u0, p, s, C, I);
    const int gt = pr->cl_gov_type[c];
    if (gt == GP_IEESGO) ieesgo_eval(ref(pr->dev[GP_IEESGO], pr->cl_gov[c]), z, p, s);
    else if (gt == GP_TGOV1) tgov1_eval(ref(pr->dev[GP_TGOV1], pr->cl_gov[c]), z, p, s);
    const int et = pr->cl_exc_type[c];
    if (et == GP_SEXS) sexs_eval(ref(pr->dev[GP_SEXS], pr->cl_exc[c]), net, z, p, s);
    else if (et == GP_ESDC1A) esdc1a_eval(ref(pr->dev[GP_ESDC1A], pr->cl_exc[c]), net, z, p, s);
    if (pr->cl_pss[c] >= 0) ieeest_eval(ref(pr->dev[GP_IEEEST], pr->cl_pss[c]), z, p, s);
}

// Minimum-cost perfect assignment (Hungarian method, O(n^3)).
std::vector<int> assign(const std::vector<std::vector<double>> &cost) {
    const int n = (int)cost.size();
    const double INF = 1e300;
    std::vector<double> u(n + 1, 0.0), v(n + 1, 0.0);
    std::vector<int> pm(n + 1, 0), way(n + 1, 0);
    for (int i = 1; i <= n; i++) {
        pm[0] = i;
        int j0 = 0;
        std::vector<double> minv(n + 1, INF);
        std::vector<char> used(n + 1, 0);
        do {
            used[j0] = 1;
            const int i0 = pm[j0];
            double delta = INF;
            int j1 = 0;
            for (int j = 1; j <= n; j++)
                if (!used[j]) {
                    const double cur = cost[i0 - 1][j - 1] - u[i0] - v[j];
                    if (cur < minv[j]) { minv[j] = cur; way[j] = j0; }
                    if (minv[j] < delta) { delta = minv[j]; j1 = j; }
                }
            for (int j = 0; j <= n; j++) {
                if (used[j]) { u[pm[j]] += delta; v[j] -= delta; }
                else minv[j] -= delta;
            }
            j0 = j1;
        } while (pm[j0] != 0);
        do {
            const int j1 = way[j0];
            pm[j0] = pm[j1];
            j0 = j1;
        } while (j0);
    }
    std::vector<int> row_to_col(n, -1);
    for (int j = 1; j <= n; j++) row_to_col[pm[j] - 1] = j - 1;
    return row_to_col;
}

}  // namespace

void make_cluster_plan(const gp_problem *pr, const double *z0, const double *u0, const double *p,
                       ClusterPlan &pl) {
    const int net = pr->n_diff + pr->n_alg;
    const int n_sys = net + 2 * pr->n_bus;
    std::vector<double> zz(n_sys, 0.0), uu(std::max(1, pr->n_ctrl), 0.0), pz(std::max(1, pr->n_par), 0.0);
    std::map<std::vector<int>, int> key_to_class;
    std::vector<std::set<int>> cls_ent;
    std::vector<std::vector<int>> cls_loc3;
    pl.cluster_class.assign(pr->n_clusters, -1);
    std::vector<std::vector<int>> members;
    for (int c = 0; c < pr->n_clusters; c++) {
        if (pr->cl_gen[c] < 0) continue;
        const int W = pr->cl_w_size[c], ws = pr->cl_w_start[c];
        std::set<int> ent;
        PatSink ps{ws, &ent};
        double C[6], I[2];
        eval_cluster(pr, c, zz.data(), uu.data(), pz.data(), ps, C, I);
        for (int r = 0; r < W; r++)
            if (pr->is_diff[ws + r]) ent.insert(r * 32 + r);
        for (int e : ent) {
            const int r = e / 32, cc = e % 32;
            if (r >= W || (cc >= W && cc < 29)) throw std::runtime_error("cluster entry outside its block");
        }
        const DevRef g = ref(pr->dev[GP_GENROU], pr->cl_gen[c]);
        std::vector<int> loc3 = {g.dp + 5 - ws, g.ap + 2 - ws, g.ap + 3 - ws};
        std::vector<int> key = {W, pr->cl_gov_type[c], pr->cl_exc_type[c], pr->cl_pss[c] >= 0 ? 1 : 0};
        for (int r = 0; r < W; r++) key.push_back(pr->is_diff[ws + r]);
        key.insert(key.end(), loc3.begin(), loc3.end());
        key.insert(key.end(), ent.begin(), ent.end());
        auto it = key_to_class.find(key);
        int cls;
        if (it == key_to_class.end()) {
            cls = (int)cls_ent.size();
            key_to_class[key] = cls;
            cls_ent.push_back(ent);
            cls_loc3.push_back(loc3);
            pl.cls_W.push_back(W);
            pl.cls_rep.push_back(c);
            members.emplace_back();
        } else {
            cls = it->second;
        }
        pl.cluster_class[c] = cls;
        members[cls].push_back(c);
    }
    pl.n_class = (int)cls_ent.size();
    pl.slot_of.assign((size_t)pl.n_class * 1024, 0);
    pl.perm_col.assign((size_t)pl.n_class * 32, 0);
    pl.pos3.assign((size_t)pl.n_class * 3, 0);
    pl.prog_ptr.assign(1, 0);
    pl.prog_mid.clear();
    pl.prog_sol.clear();
    pl.rhs_base.clear();
    pl.nslot.clear();
    pl.ops.clear();
    pl.max_slots = 0;
    pl.lu_flops = 0;
    const double dt_rep = 1.0 / 120.0;
    for (int cls = 0; cls < pl.n_class; cls++) {
        const int W = pl.cls_W[cls], rep = pl.cls_rep[cls], ws = pr->cl_w_start[rep];
        const std::set<int> &ent = cls_ent[cls];
        std::vector<std::vector<char>> pat(W, std::vector<char>(W, 0));
        for (int e : ent)
            if (e % 32 < W) pat[e / 32][e % 32] = 1;
        // representative values (scenario 0) with the backward-Euler scaling
        std::vector<double> a(1024, 0.0);
        DenseSink ds{ws, a.data()};
        double C[6], I[2];
        eval_cluster(pr, rep, z0, u0, p, ds, C, I);
        std::vector<char> isd(W);
        for (int r = 0; r < W; r++) {
            isd[r] = pr->is_diff[ws + r] ? 1 : 0;
            if (isd[r]) {
                for (int c = 0; c < W; c++) a[r * 32 + c] *= -dt_rep;
                a[r * 32 + r] += 1.0;
            }
        }
        // pivot pairs: differential rows keep their diagonal, algebraic rows
        // are matched to algebraic columns by maximum product of |a_ij|
        std::vector<int> alg;
        for (int r = 0; r < W; r++)
            if (!isd[r]) alg.push_back(r);
        std::vector<int> row_of_col(W);
        for (int r = 0; r < W; r++)
            if (isd[r]) row_of_col[r] = r;
        if (!alg.empty()) {
            const int na = (int)alg.size();
            std::vector<std::vector<double>> cost(na, std::vector<double>(na, 1e30));
            for (int i = 0; i < na; i++)
                for (int j = 0; j < na; j++)
                    if (pat[alg[i]][alg[j]]) {
                        const double v = std::fabs(a[alg[i] * 32 + alg[j]]);
                        cost[i][j] = v > 0.0 ? -std::log(v) : 700.0;
                    }
            std::vector<int> r2c = assign(cost);
            for (int i = 0; i < na; i++) {
                if (!pat[alg[i]][alg[r2c[i]]])
                    throw std::runtime_error("cluster block has no structurally non-singular pivot choice");
                row_of_col[alg[r2c[i]]] = alg[i];
            }
        }
        // minimum-degree order of the pivot pairs (indexed by column)
        std::vector<std::vector<char>> G(W, std::vector<char>(W, 0));
        for (int i = 0; i < W; i++)
            for (int j = 0; j < W; j++)
                if (i != j && pat[row_of_col[i]][j]) G[i][j] = G[j][i] = 1;
        std::vector<int> ord;
        std::vector<char> alive(W, 1);
        for (int step = 0; step < W; step++) {
            int best = -1, bd = 1 << 30;
            for (int v = 0; v < W; v++)
                if (alive[v]) {
                    int dgr = 0;
                    for (int u = 0; u < W; u++) dgr += alive[u] && G[v][u];
                    if (dgr < bd) { bd = dgr; best = v; }
                }
            ord.push_back(best);
            alive[best] = 0;
            for (int x = 0; x < W; x++)
                if (alive[x] && G[best][x])
                    for (int y = 0; y < W; y++)
                        if (alive[y] && G[best][y] && x != y) G[x][y] = 1;
        }
        std::vector<int> ipcol(W), iprow(W);
        for (int k = 0; k < W; k++) {
            ipcol[ord[k]] = k;
            iprow[row_of_col[ord[k]]] = k;
        }
        // symbolic LU of the permuted block
        std::vector<std::vector<char>> Q(W, std::vector<char>(W, 0));
        for (int r = 0; r < W; r++)
            for (int c = 0; c < W; c++)
                if (pat[r][c]) Q[iprow[r]][ipcol[c]] = 1;
        for (int k = 0; k < W; k++) {
            if (!Q[k][k]) throw std::runtime_error("zero structural pivot in a cluster block");
            for (int i = k + 1; i < W; i++)
                if (Q[i][k])
                    for (int j = k + 1; j < W; j++)
                        if (Q[k][j]) Q[i][j] = 1;
        }
        std::vector<std::vector<int>> slot(W, std::vector<int>(W, -1));
        int ns = 0;
        for (int i = 0; i < W; i++)
            for (int j = 0; j < W; j++)
                if (Q[i][j]) slot[i][j] = ns++;
        const int inv0 = ns;
        const int rb = inv0 + W;
        const int trash = rb + 3 * W;
        const int nslot = trash + 1;
        short *so = pl.slot_of.data() + (size_t)cls * 1024;
        for (int q = 0; q < 1024; q++) so[q] = (short)trash;
        for (int r = 0; r < W; r++) {
            for (int c = 0; c < W; c++)
                if (slot[iprow[r]][ipcol[c]] >= 0) so[r * 32 + c] = (short)slot[iprow[r]][ipcol[c]];
            so[r * 32 + 29] = (short)(rb + iprow[r]);
            so[r * 32 + 30] = (short)(rb + W + iprow[r]);
            so[r * 32 + 31] = (short)(rb + 2 * W + iprow[r]);
        }
        auto op = [&](unsigned char code, int d, int a_, int b) {
            CluOp o;
            o.code = code;
            o.pad = 0;
            o.d = (short)d;
            o.a = (short)a_;
            o.b = (short)b;
            pl.ops.push_back(o);
        };
        // part 1: backward-Euler scaling of the differential rows
        for (int r = 0; r < W; r++) {
            if (!isd[r]) {
                op(OP_ROW, rb + 2 * W + iprow[r], r, 0);
                continue;
            }
            for (int c = 0; c < W; c++)
                if (ent.count(r * 32 + c)) op(OP_SCL, slot[iprow[r]][ipcol[c]], 0, 0);
            if (ent.count(r * 32 + 29)) op(OP_SCL, rb + iprow[r], 0, 0);
            if (ent.count(r * 32 + 30)) op(OP_SCL, rb + W + iprow[r], 0, 0);
            op(OP_DIAG, slot[iprow[r]][ipcol[r]], 0, 0);
            op(OP_BEF, rb + 2 * W + iprow[r], r, 0);
        }
        pl.prog_mid.push_back((int)pl.ops.size());
        // part 2: LU without pivoting on the permuted block, then the solves
        int64_t fl = 0;
        for (int k = 0; k < W; k++) {
            op(OP_RCP, inv0 + k, slot[k][k], 0);
            for (int i = k + 1; i < W; i++)
                if (Q[i][k]) op(OP_MUL, slot[i][k], inv0 + k, 0);
            for (int i = k + 1; i < W; i++)
                if (Q[i][k])
                    for (int j = k + 1; j < W; j++)
                        if (Q[k][j]) { op(OP_FMS, slot[i][j], slot[i][k], slot[k][j]); fl++; }
        }
        pl.prog_sol.push_back((int)pl.ops.size());
        for (int k = 0; k < W; k++)
            for (int i = k + 1; i < W; i++)
                if (Q[i][k]) { op(OP_FMS3, i, slot[i][k], k); fl += 3; }
        for (int k = W - 1; k >= 0; k--) {
            op(OP_MUL3, k, inv0 + k, 0);
            for (int i = 0; i < k; i++)
                if (Q[i][k]) { op(OP_FMS3, i, slot[i][k], k); fl += 3; }
        }
        pl.prog_ptr.push_back((int)pl.ops.size());
        pl.rhs_base.push_back(rb);
        pl.nslot.push_back(nslot);
        pl.max_slots = std::max(pl.max_slots, nslot);
        for (int j = 0; j < W; j++) pl.perm_col[(size_t)cls * 32 + j] = ord[j];
        for (int t = 0; t < 3; t++) pl.pos3[(size_t)cls * 3 + t] = ipcol[cls_loc3[cls][t]];
        pl.lu_flops += fl * (int64_t)members[cls].size();
    }
    // warp tasks: 32 clusters of one class, the classes with the most slots
    // (the longest programs) first, so that the warps that start last are
    // the short ones
    pl.order.clear();
    pl.task_class.clear();
    pl.task_first.clear();
    pl.task_count.clear();
    std::vector<int> by_len(pl.n_class);
    for (int cls = 0; cls < pl.n_class; cls++) by_len[cls] = cls;
    std::stable_sort(by_len.begin(), by_len.end(), [&](int a, int b) { return pl.nslot[a] > pl.nslot[b]; });
    for (int cls : by_len) {
        const int first = (int)pl.order.size();
        pl.order.insert(pl.order.end(), members[cls].begin(), members[cls].end());
        for (size_t s = 0; s < members[cls].size(); s += 32) {
            pl.task_class.push_back(cls);
            pl.task_first.push_back(first + (int)s);
            pl.task_count.push_back((int)std::min<size_t>(32, members[cls].size() - s));
        }
    }
}

double host_cluster_run(const gp_problem *pr, const ClusterPlan &pl, int c, const double *z, const double *zold,
                        const double *u0, const double *p, double dt, double *yx, double *out8, double *f_out) {
    const int cls = pl.cluster_class[c];
    if (cls < 0) throw std::runtime_error("trivial cluster has no program");
    const int W = pl.cls_W[cls], ws = pr->cl_w_start[c];
    std::vector<double> v(pl.nslot[cls], 0.0);
    SlotSink s{ws, pl.slot_of.data() + (size_t)cls * 1024, v.data()};
    double C[6], I[2];
    eval_cluster(pr, c, z, u0, p, s, C, I);
    const int rb = pl.rhs_base[cls];
    double *R0 = v.data() + rb, *R1 = R0 + W, *R2 = R1 + W;
    for (int q = pl.prog_ptr[cls]; q < pl.prog_mid[cls]; q++) {
        const CluOp &o = pl.ops[q];
        if (o.code == OP_SCL) v[o.d] *= -dt;
        else if (o.code == OP_DIAG) v[o.d] += 1.0;
        else if (o.code == OP_BEF) v[o.d] = z[ws + o.a] - zold[ws + o.a] - dt * v[o.d];
        if ((o.code == OP_BEF || o.code == OP_ROW) && f_out) f_out[o.a] = v[o.d];
    }
    double fmax = 0.0;
    for (int j = 0; j < W; j++) fmax = std::max(fmax, std::fabs(R2[j]));
    for (int q = pl.prog_mid[cls]; q < pl.prog_ptr[cls + 1]; q++) {
        const CluOp &o = pl.ops[q];
        switch (o.code) {
        case OP_RCP: v[o.d] = 1.0 / v[o.a]; break;
        case OP_MUL: v[o.d] *= v[o.a]; break;
        case OP_FMS: v[o.d] -= v[o.a] * v[o.b]; break;
        case OP_FMS3: {
            const double l = v[o.a];
            R0[o.d] -= l * R0[o.b];
            R1[o.d] -= l * R1[o.b];
            R2[o.d] -= l * R2[o.b];
            break;
        }
        case OP_MUL3: {
            const double l = v[o.a];
            R0[o.d] *= l;
            R1[o.d] *= l;
            R2[o.d] *= l;
            break;
        }
        default: break;
        }
    }
    for (int j = 0; j < W; j++) {
        const int st = pl.perm_col[(size_t)cls * 32 + j];
        yx[st] = R2[j];
        yx[W + st] = R0[j];
        yx[2 * W + st] = R1[j];
    }
    const int *p3 = pl.pos3.data() + (size_t)cls * 3;
    double X1[3], X2[3], Y[3];
    for (int t = 0; t < 3; t++) {
        X1[t] = R0[p3[t]];
        X2[t] = R1[p3[t]];
        Y[t] = R2[p3[t]];
    }
    out8[0] = C[0] * X1[0] + C[1] * X1[1] + C[2] * X1[2];
    out8[1] = C[0] * X2[0] + C[1] * X2[1] + C[2] * X2[2];
    out8[2] = C[3] * X1[0] + C[4] * X1[1] + C[5] * X1[2];
    out8[3] = C[3] * X2[0] + C[4] * X2[1] + C[5] * X2[2];
    out8[4] = C[0] * Y[0] + C[1] * Y[1] + C[2] * Y[2];
    out8[5] = C[3] * Y[0] + C[4] * Y[1] + C[5] * Y[2];
    out8[6] = I[0];
    out8[7] = I[1];
    return fmax;
}

}  // namespace gp
