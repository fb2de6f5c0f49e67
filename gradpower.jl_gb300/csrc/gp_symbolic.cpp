// Host-once symbolic analysis: nested dissection on the bus graph, the
// elimination tree, fundamental supernodes, multifrontal front layout and
// the level schedule.  See gp_symbolic.h.
#include "gp_symbolic.h"

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <queue>
#include <stdexcept>

namespace gp {
namespace {

struct Graph {
    int n = 0;
    std::vector<int> ptr, adj;
};

// Minimum-degree order of a small induced subgraph (|V| <= 64) using an
// explicit elimination graph held in 64-bit masks.
void leaf_min_degree(const Graph &G, const std::vector<int> &V, std::vector<int> &pos_in,
                     std::vector<int> &order) {
    const int k = (int)V.size();
    for (int a = 0; a < k; a++) pos_in[V[a]] = a;
    std::vector<uint64_t> m(k, 0);
    for (int a = 0; a < k; a++) {
        int v = V[a];
        for (int q = G.ptr[v]; q < G.ptr[v + 1]; q++) {
            int b = pos_in[G.adj[q]];
            if (b >= 0 && b != a) m[a] |= (uint64_t)1 << b;
        }
    }
    uint64_t alive = (k == 64) ? ~(uint64_t)0 : (((uint64_t)1 << k) - 1);
    for (int step = 0; step < k; step++) {
        int best = -1, bd = 1 << 30;
        for (int a = 0; a < k; a++)
            if (alive >> a & 1) {
                int d = __builtin_popcountll(m[a] & alive);
                if (d < bd) { bd = d; best = a; }
            }
        uint64_t nb = m[best] & alive & ~((uint64_t)1 << best);
        for (int a = 0; a < k; a++)
            if (nb >> a & 1) m[a] |= nb & ~((uint64_t)1 << a);
        alive &= ~((uint64_t)1 << best);
        order.push_back(V[best]);
    }
    for (int a = 0; a < k; a++) pos_in[V[a]] = -1;
}

struct ND {
    const Graph &G;
    std::vector<int> set_id, lev, pos_in;
    std::vector<int> order;
    int next_id = 1;
    static constexpr int LEAF = 48;

    explicit ND(const Graph &g) : G(g), set_id(g.n, 0), lev(g.n, -1), pos_in(g.n, -1) {}

    // BFS inside the set `sid` from r; fills lev for visited nodes and
    // returns the visited nodes in BFS order.
    void bfs(int r, int sid, std::vector<int> &visit) {
        visit.clear();
        visit.push_back(r);
        lev[r] = 0;
        for (size_t h = 0; h < visit.size(); h++) {
            int u = visit[h];
            for (int q = G.ptr[u]; q < G.ptr[u + 1]; q++) {
                int v = G.adj[q];
                if (set_id[v] == sid && lev[v] < 0) {
                    lev[v] = lev[u] + 1;
                    visit.push_back(v);
                }
            }
        }
    }

    void clear_lev(const std::vector<int> &V) {
        for (int v : V) lev[v] = -1;
    }

    void run(std::vector<int> V, int sid) {
        if ((int)V.size() <= LEAF) {
            leaf_min_degree(G, V, pos_in, order);
            return;
        }
        // connected components
        std::vector<int> visit;
        bfs(V[0], sid, visit);
        if (visit.size() < V.size()) {
            std::vector<std::vector<int>> comps;
            comps.push_back(visit);
            for (int v : V)
                if (lev[v] < 0) {
                    std::vector<int> c;
                    bfs(v, sid, c);
                    comps.push_back(c);
                }
            clear_lev(V);
            for (auto &c : comps) {
                int id = next_id++;
                for (int v : c) set_id[v] = id;
                run(c, id);
            }
            return;
        }
        // pseudo-peripheral start: repeat BFS from a farthest, lowest-degree node
        int r = V[0];
        int depth = -1;
        for (int t = 0; t < 4; t++) {
            clear_lev(V);
            bfs(r, sid, visit);
            int d = lev[visit.back()];
            if (d <= depth) break;
            depth = d;
            int best = visit.back(), bd = 1 << 30;
            for (int i = (int)visit.size() - 1; i >= 0 && lev[visit[i]] == d; i--) {
                int v = visit[i];
                int dg = 0;
                for (int q = G.ptr[v]; q < G.ptr[v + 1]; q++) dg += set_id[G.adj[q]] == sid;
                if (dg < bd) { bd = dg; best = v; }
            }
            r = best;
        }
        clear_lev(V);
        bfs(r, sid, visit);
        int nlev = lev[visit.back()] + 1;
        std::vector<int> cnt(nlev + 1, 0);
        for (int v : V) cnt[lev[v]]++;
        int half = (int)V.size() / 2, acc = 0, l = 0;
        for (l = 0; l < nlev; l++) {
            acc += cnt[l];
            if (acc >= half) break;
        }
        if (l >= nlev - 1) l = std::max(0, nlev - 2);
        std::vector<int> A, B, S;
        for (int v : V) {
            if (lev[v] < l) A.push_back(v);
            else if (lev[v] > l) B.push_back(v);
            else {
                bool touches = false;
                for (int q = G.ptr[v]; q < G.ptr[v + 1] && !touches; q++) {
                    int u = G.adj[q];
                    touches = set_id[u] == sid && lev[u] == l + 1;
                }
                (touches ? S : A).push_back(v);
            }
        }
        clear_lev(V);
        if (A.empty() || B.empty()) {
            // no useful split: order the whole set by minimum degree on its
            // own adjacency (ties in BFS order)
            std::vector<int> tmp = V;
            while (!tmp.empty()) {
                size_t take = std::min<size_t>(LEAF, tmp.size());
                std::vector<int> chunk(tmp.begin(), tmp.begin() + take);
                leaf_min_degree(G, chunk, pos_in, order);
                tmp.erase(tmp.begin(), tmp.begin() + take);
            }
            return;
        }
        int ida = next_id++, idb = next_id++, ids = next_id++;
        for (int v : A) set_id[v] = ida;
        for (int v : B) set_id[v] = idb;
        for (int v : S) set_id[v] = ids;
        run(A, ida);
        run(B, idb);
        // separator nodes: order them by minimum degree in chunks
        for (size_t a = 0; a < S.size(); a += LEAF) {
            std::vector<int> chunk(S.begin() + a, S.begin() + std::min(S.size(), a + LEAF));
            leaf_min_degree(G, chunk, pos_in, order);
        }
    }
};

void merge_into(std::vector<int> &dst, const std::vector<int> &src, int skip_le) {
    // dst := dst ∪ {x in src : x > skip_le}, both sorted
    std::vector<int> out;
    out.reserve(dst.size() + src.size());
    size_t i = 0, j = 0;
    while (j < src.size() && src[j] <= skip_le) j++;
    while (i < dst.size() || j < src.size()) {
        int x;
        if (j >= src.size() || (i < dst.size() && dst[i] < src[j])) x = dst[i++];
        else if (i >= dst.size() || src[j] < dst[i]) x = src[j++];
        else { x = dst[i++]; j++; }
        out.push_back(x);
    }
    dst.swap(out);
}

}  // namespace

void analyse(int n, const std::vector<int> &rowptr, const std::vector<int> &colidx,
             const std::vector<int> &group, int n_nodes, Symbolic &S) {
    // ---- node graph ----
    Graph G;
    G.n = n_nodes;
    {
        std::vector<std::vector<int>> nb(n_nodes);
        for (int i = 0; i < n; i++)
            for (int q = rowptr[i]; q < rowptr[i + 1]; q++) {
                int a = group[i], b = group[colidx[q]];
                if (a != b) { nb[a].push_back(b); nb[b].push_back(a); }
            }
        G.ptr.assign(n_nodes + 1, 0);
        for (int a = 0; a < n_nodes; a++) {
            std::sort(nb[a].begin(), nb[a].end());
            nb[a].erase(std::unique(nb[a].begin(), nb[a].end()), nb[a].end());
            G.ptr[a + 1] = G.ptr[a] + (int)nb[a].size();
        }
        G.adj.reserve(G.ptr[n_nodes]);
        for (int a = 0; a < n_nodes; a++) G.adj.insert(G.adj.end(), nb[a].begin(), nb[a].end());
    }
    // ---- nested dissection on nodes ----
    ND nd(G);
    {
        std::vector<int> all(n_nodes);
        for (int a = 0; a < n_nodes; a++) all[a] = a;
        nd.run(all, 0);
    }
    if ((int)nd.order.size() != n_nodes) throw std::runtime_error("nested dissection lost nodes");
    // ---- expand to scalar unknowns ----
    std::vector<std::vector<int>> members(n_nodes);
    for (int i = 0; i < n; i++) members[group[i]].push_back(i);
    S.n = n;
    S.perm.clear();
    S.perm.reserve(n);
    for (int a : nd.order)
        for (int i : members[a]) S.perm.push_back(i);
    if ((int)S.perm.size() != n) throw std::runtime_error("unknowns without a node");
    S.iperm.assign(n, 0);
    for (int k = 0; k < n; k++) S.iperm[S.perm[k]] = k;
    // ---- permuted symmetric pattern: lower part per column ----
    std::vector<std::vector<int>> low(n), upp(n);
    for (int i = 0; i < n; i++)
        for (int q = rowptr[i]; q < rowptr[i + 1]; q++) {
            int a = S.iperm[i], b = S.iperm[colidx[q]];
            if (a == b) continue;
            int lo = std::min(a, b), hi = std::max(a, b);
            low[lo].push_back(hi);
            upp[hi].push_back(lo);
        }
    for (int j = 0; j < n; j++) {
        std::sort(low[j].begin(), low[j].end());
        low[j].erase(std::unique(low[j].begin(), low[j].end()), low[j].end());
        std::sort(upp[j].begin(), upp[j].end());
        upp[j].erase(std::unique(upp[j].begin(), upp[j].end()), upp[j].end());
    }
    // ---- elimination tree (Liu, path compression) ----
    std::vector<int> par(n, -1), anc(n, -1);
    for (int j = 0; j < n; j++)
        for (int i : upp[j]) {
            int r = i;
            while (anc[r] != -1 && anc[r] != j) {
                int nx = anc[r];
                anc[r] = j;
                r = nx;
            }
            if (anc[r] == -1) { anc[r] = j; par[r] = j; }
        }
    // ---- column structures ----
    std::vector<int> nchild(n, 0);
    for (int j = 0; j < n; j++)
        if (par[j] >= 0) nchild[par[j]]++;
    std::vector<std::vector<int>> cs(n);
    std::vector<std::vector<int>> kids(n);
    for (int j = 0; j < n; j++)
        if (par[j] >= 0) kids[par[j]].push_back(j);
    for (int j = 0; j < n; j++) {
        cs[j] = low[j];
        for (int c : kids[j]) merge_into(cs[j], cs[c], j);
    }
    // ---- fundamental supernodes ----
    std::vector<int> fstart;
    for (int j = 0; j < n; j++) {
        bool join = j > 0 && par[j - 1] == j && nchild[j] == 1 && cs[j - 1].size() == cs[j].size() + 1;
        if (!join) fstart.push_back(j);
    }
    int nf = (int)fstart.size();
    fstart.push_back(n);
    // ---- amalgamation: merge a supernode into its parent when the
    // parent's columns follow it directly and the merge adds at most
    // `relax_zeros` explicit zeros (0 = only exact nesting) ----
    {
        std::vector<int> fsup_of(n);
        for (int f = 0; f < nf; f++)
            for (int j = fstart[f]; j < fstart[f + 1]; j++) fsup_of[j] = f;
        std::vector<int> st(fstart.begin(), fstart.end() - 1), ncol(nf), fpar(nf, -1);
        std::vector<char> gone(nf, 0);
        for (int f = 0; f < nf; f++) {
            ncol[f] = fstart[f + 1] - fstart[f];
            int last = fstart[f + 1] - 1;
            if (par[last] >= 0) fpar[f] = fsup_of[par[last]];
        }
        for (int f = 0; f < nf; f++) {
            int p = fpar[f];
            if (p < 0 || fstart[f + 1] != st[p]) continue;
            int64_t rs = (int64_t)cs[fstart[f + 1] - 1].size();
            int64_t rp = (int64_t)cs[fstart[p + 1] - 1].size();
            int64_t extra = (int64_t)ncol[f] * (ncol[p] + rp - rs);
            int64_t width = ncol[f] + ncol[p];
            bool ok = extra == 0 || (width <= 48 && extra <= width * 2);
            if (!ok) continue;
            st[p] = st[f];
            ncol[p] += ncol[f];
            gone[f] = 1;
        }
        S.sup_start.clear();
        for (int f = 0; f < nf; f++)
            if (!gone[f]) S.sup_start.push_back(st[f]);
        std::sort(S.sup_start.begin(), S.sup_start.end());
    }
    S.nsup = (int)S.sup_start.size();
    S.sup_start.push_back(n);
    S.sup_of.assign(n, 0);
    for (int s = 0; s < S.nsup; s++)
        for (int j = S.sup_start[s]; j < S.sup_start[s + 1]; j++) S.sup_of[j] = s;
    S.row_ptr.assign(S.nsup + 1, 0);
    S.rows.clear();
    for (int s = 0; s < S.nsup; s++) {
        int last = S.sup_start[s + 1] - 1;
        S.rows.insert(S.rows.end(), cs[last].begin(), cs[last].end());
        S.row_ptr[s + 1] = (int)S.rows.size();
    }
    S.parent.assign(S.nsup, -1);
    for (int s = 0; s < S.nsup; s++) {
        int last = S.sup_start[s + 1] - 1;
        if (par[last] >= 0) S.parent[s] = S.sup_of[par[last]];
    }
    // children
    std::vector<int> ccount(S.nsup + 1, 0);
    for (int s = 0; s < S.nsup; s++)
        if (S.parent[s] >= 0) ccount[S.parent[s] + 1]++;
    S.child_ptr.assign(S.nsup + 1, 0);
    for (int s = 0; s < S.nsup; s++) S.child_ptr[s + 1] = S.child_ptr[s] + ccount[s + 1];
    S.children.assign(S.child_ptr[S.nsup], 0);
    {
        std::vector<int> fill(S.child_ptr.begin(), S.child_ptr.end() - 1);
        for (int s = 0; s < S.nsup; s++)
            if (S.parent[s] >= 0) S.children[fill[S.parent[s]]++] = s;
    }
    // levels (children have smaller indices than parents)
    S.level.assign(S.nsup, 0);
    S.nlevels = 0;
    for (int s = 0; s < S.nsup; s++) {
        int lv = 0;
        for (int q = S.child_ptr[s]; q < S.child_ptr[s + 1]; q++) lv = std::max(lv, S.level[S.children[q]] + 1);
        S.level[s] = lv;
        S.nlevels = std::max(S.nlevels, lv + 1);
    }
    S.level_ptr.assign(S.nlevels + 1, 0);
    for (int s = 0; s < S.nsup; s++) S.level_ptr[S.level[s] + 1]++;
    for (int l = 0; l < S.nlevels; l++) S.level_ptr[l + 1] += S.level_ptr[l];
    S.level_sups.assign(S.nsup, 0);
    {
        std::vector<int> fill(S.level_ptr.begin(), S.level_ptr.end() - 1);
        for (int s = 0; s < S.nsup; s++) S.level_sups[fill[S.level[s]]++] = s;
    }
    // fronts, update vectors, relative maps, costs
    S.front_off.assign(S.nsup + 1, 0);
    S.uvec_off.assign(S.nsup + 1, 0);
    S.relmap_ptr.assign(S.nsup + 1, 0);
    S.nnz_lu = 0;
    S.flops = 0.0;
    S.max_front = 0;
    for (int s = 0; s < S.nsup; s++) {
        int m = S.front_m(s), ns = S.front_n(s), r = S.front_r(s);
        S.front_off[s + 1] = S.front_off[s] + (int64_t)m * m;
        S.uvec_off[s + 1] = S.uvec_off[s] + r;
        S.relmap_ptr[s + 1] = S.relmap_ptr[s] + r;
        S.nnz_lu += (int64_t)ns * ns + 2LL * ns * r;
        for (int k = 0; k < ns; k++) {
            double t = m - k - 1;
            S.flops += t + 2.0 * t * t;
        }
        S.max_front = std::max(S.max_front, m);
    }
    S.relmap.assign(S.relmap_ptr[S.nsup], 0);
    for (int c = 0; c < S.nsup; c++) {
        int s = S.parent[c];
        int base = S.relmap_ptr[c];
        for (int a = 0; a < S.front_r(c); a++) {
            int i = S.rows[S.row_ptr[c] + a];
            if (s < 0) throw std::runtime_error("root supernode with a non-empty row structure");
            int pos;
            if (i < S.sup_start[s + 1]) {
                pos = i - S.sup_start[s];
                if (pos < 0) throw std::runtime_error("relative index below parent");
            } else {
                auto b = S.rows.begin() + S.row_ptr[s], e = S.rows.begin() + S.row_ptr[s + 1];
                auto it = std::lower_bound(b, e, i);
                if (it == e || *it != i) throw std::runtime_error("child row missing from parent structure");
                pos = S.front_n(s) + (int)(it - b);
            }
            S.relmap[base + a] = pos;
        }
    }
}

}  // namespace gp
