// Block-size configuration and GPS-style bandwidth reordering.
//
// The ordering decides the block sparsity pattern and hence the whole op DAG,
// so it follows the reference's choices step for step (GPSOrder.cpp:41-650),
// including its candidate sampling and the tie-breaking of its sorts, which
// are reproduced by sorting the same sequences with the same key.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <set>
#include <stdexcept>
#include <vector>

#include "plan.h"

namespace sog {

// config.cpp:30-49: block rows = smallest power of two strictly greater than
// n/64; coarse rows = 2 << (popcount(block_rows-1)/2).
Config make_config(int n) {
    Config c;
    c.n = n;
    int m = n / 64, r = 1;
    while (m > 0) { m /= 2; r *= 2; }
    if (r < 2) r = 2;  // n < 64 is padded to two block rows (the reference divides by zero there)
    c.block_rows = r;
    c.block_rows_l2 = 2 << (__builtin_popcount((unsigned)(r - 1)) / 2);
    c.block_size_l2 = 64 * r / c.block_rows_l2;
    return c;
}

namespace {

// Symmetrised adjacency without self loops, each row sorted and unique
// (GPSOrder.cpp:279-338).
struct Graph {
    int n = 0;
    std::vector<int32_t> ptr, adj;
    int deg(int v) const { return ptr[v + 1] - ptr[v]; }
    const int32_t* begin(int v) const { return adj.data() + ptr[v]; }
    const int32_t* end(int v) const { return adj.data() + ptr[v + 1]; }
};

Graph build_graph(int n, const std::vector<int32_t>& I, const std::vector<int32_t>& J) {
    Graph g;
    g.n = n;
    std::vector<int32_t> cnt(n + 1, 0);
    for (size_t k = 0; k < I.size(); k++)
        if (I[k] != J[k]) { cnt[I[k]]++; cnt[J[k]]++; }
    std::vector<int32_t> ptr(n + 1, 0);
    for (int i = 0; i < n; i++) ptr[i + 1] = ptr[i] + cnt[i];
    std::vector<int32_t> tmp(ptr[n]);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (size_t k = 0; k < I.size(); k++)
        if (I[k] != J[k]) { tmp[fill[I[k]]++] = J[k]; tmp[fill[J[k]]++] = I[k]; }
    g.ptr.assign(n + 1, 0);
    g.adj.reserve(tmp.size());
    for (int i = 0; i < n; i++) {
        std::sort(tmp.begin() + ptr[i], tmp.begin() + ptr[i + 1]);
        int32_t last = -1;
        for (int32_t k = ptr[i]; k < ptr[i + 1]; k++) {
            if (k > ptr[i] && tmp[k] == last) continue;
            g.adj.push_back(tmp[k]);
            last = tmp[k];
        }
        g.ptr[i + 1] = (int32_t)g.adj.size();
    }
    return g;
}

using Levels = std::vector<std::vector<int32_t>>;

// Breadth-first level structure from `start`; nodes not reached are added as
// further components, each rooted at the smallest unreached node
// (GPSOrder.cpp:185-277).
Levels level_structure(const Graph& g, int start) {
    Levels lv;
    std::vector<char> seen(g.n, 0);
    auto bfs_from = [&](int root) {
        lv.push_back({root});
        seen[root] = 1;
        for (;;) {
            const std::vector<int32_t>& cur = lv.back();
            std::vector<int32_t> nxt;
            for (int32_t v : cur)
                for (const int32_t* p = g.begin(v); p != g.end(v); ++p)
                    if (!seen[*p]) { seen[*p] = 1; nxt.push_back(*p); }
            if (nxt.empty()) break;
            lv.push_back(std::move(nxt));
        }
    };
    bfs_from(start);
    int scan = 0;
    for (;;) {
        while (scan < g.n && seen[scan]) scan++;
        if (scan >= g.n) break;
        bfs_from(scan);
    }
    return lv;
}

int width_of(const Levels& lv) {
    size_t w = 0;
    for (auto& l : lv) w = std::max(w, l.size());
    return (int)w;
}

struct Ranked {
    int32_t index, value;
};
inline bool by_value(const Ranked& x, const Ranked& y) { return x.value < y.value; }
inline bool by_value_desc(const Ranked& x, const Ranked& y) { return y.value < x.value; }

// Numbering along a level structure (GPSOrder.cpp:340-450). `alive` marks,
// for node w and each neighbour slot, whether that neighbour is still in w's
// to-be-done set; a neighbour is removed from the sets of already-numbered
// nodes once it is numbered itself.
struct Numbering {
    const Graph& g;
    std::vector<int32_t> nsum;  // sum of neighbour degrees
    std::vector<char> alive;
    std::vector<int32_t> alive_cnt;
    std::vector<int32_t> new_of, old_of;
    int cursor = 0;

    explicit Numbering(const Graph& gr) : g(gr) {
        nsum.assign(g.n, 0);
        for (int v = 0; v < g.n; v++) {
            int s = 0;
            for (const int32_t* p = g.begin(v); p != g.end(v); ++p) s += g.deg(*p);
            nsum[v] = s;
        }
        alive.assign(g.adj.size(), 1);
        alive_cnt.resize(g.n);
        for (int v = 0; v < g.n; v++) alive_cnt[v] = g.deg(v);
        new_of.assign(g.n, -1);
        old_of.assign(g.n, -1);
    }
    void erase_from(int w, int node) {
        const int32_t* b = g.begin(w);
        const int32_t* e = g.end(w);
        const int32_t* p = std::lower_bound(b, e, node);
        if (p != e && *p == node) {
            size_t slot = p - g.adj.data();
            if (alive[slot]) { alive[slot] = 0; alive_cnt[w]--; }
        }
    }
    void number(int node) {
        new_of[node] = cursor;
        old_of[cursor] = node;
        cursor++;
        for (const int32_t* p = g.begin(node); p != g.end(node); ++p)
            if (new_of[*p] >= 0 && alive_cnt[*p] > 0) erase_from(*p, node);
    }
    void number_sorted(std::vector<Ranked>& r) {
        std::sort(r.begin(), r.end(), by_value);
        for (auto& x : r) number(x.index);
    }
    void next_level(const std::vector<int32_t>& last, const std::vector<int32_t>& cur) {
        int start = cursor;
        std::vector<Ranked> order;
        order.reserve(last.size());
        for (int32_t s : last) order.push_back({s, new_of[s]});
        std::sort(order.begin(), order.end(), by_value_desc);
        std::vector<Ranked> rank;
        for (int i = (int)order.size() - 1; i >= 0; i--) {
            int w = order[i].index;
            if (alive_cnt[w] == 0) continue;
            rank.clear();
            for (int32_t k = g.ptr[w]; k < g.ptr[w + 1]; k++) {
                if (!alive[k]) continue;
                int node = g.adj[k];
                if (new_of[node] < 0) rank.push_back({node, nsum[node]});
            }
            if (rank.empty()) continue;
            number_sorted(rank);
        }
        if (cursor - start != (int)cur.size()) {
            std::vector<Ranked> rest;
            for (int32_t v : cur)
                if (new_of[v] < 0) rest.push_back({v, nsum[v]});
            number_sorted(rest);
        }
    }
};

}  // namespace

Ordering gps_order(int n, const std::vector<int32_t>& I, const std::vector<int32_t>& J,
                   const std::vector<double>& V, int threads) {
    Ordering ord;
    Graph g = build_graph(n, I, J);
    if (threads > 0) omp_set_num_threads(threads);

    // least-connected start node (GPSOrder.cpp:464-478)
    int start = 0, best = n;
    for (int i = 0; i < n; i++) {
        int d = g.deg(i);
        if (d < best && d != 0) { start = i; best = d; }
    }
    Levels levels = level_structure(g, start);
    std::set<int32_t> gset(levels.back().begin(), levels.back().end());
    for (int v = 0; v < n; v++)
        if (g.deg(v) == g.deg(start)) gset.insert(v);

    // pseudo-peripheral search over (a sample of) the last level (GPSOrder.cpp:508-576)
    std::vector<int32_t> cand;
    std::vector<int> cand_depth, cand_width;
    for (;;) {
        const std::vector<int32_t>& last = levels.back();
        int lastsize = (int)last.size();
        int skip = 0;
        if (lastsize > 100) { skip = (lastsize + 99) / 100; skip = (skip / 2 + 1) * 2 - 1; }
        cand.clear();
        for (int t = 0; t < lastsize; t++) {
            if (skip > 0 && t % skip != 0) continue;
            cand.push_back(last[t]);
        }
        int cn = (int)cand.size();
        std::vector<Levels> lvs(cn);
#pragma omp parallel for schedule(dynamic)
        for (int t = 0; t < cn; t++) lvs[t] = level_structure(g, cand[t]);
        bool updated = false;
        int depth = (int)levels.size();
        cand_depth.assign(cn, 0);
        cand_width.assign(cn, 0);
        for (int t = 0; t < cn; t++) {
            cand_depth[t] = (int)lvs[t].size();
            cand_width[t] = width_of(lvs[t]);
        }
        for (int t = 0; t < cn; t++) {
            if ((int)lvs[t].size() < depth) continue;
            gset.insert(lvs[t].back().begin(), lvs[t].back().end());
            if ((int)lvs[t].size() > depth) {
                levels = std::move(lvs[t]);
                start = cand[t];
                updated = true;
                break;
            }
        }
        if (!updated) break;
    }

    // widen the candidate set with low-degree nodes of Gset (GPSOrder.cpp:580-612)
    int vdeg = g.deg(start);
    gset.insert(n - 1);
    gset.insert(0);
    const int LIST = 500;
    int ncand0 = (int)cand.size();
    int index = ncand0, skip = 0, cap = LIST - ncand0;
    if (cap > 0) { skip = ((int)gset.size() + cap - 1) / cap; skip = (skip / 2 + 1) * 2 - 1; }
    std::vector<int32_t> extra;
    for (int32_t s : gset) {
        if (g.deg(s) > vdeg && s != n - 1 && s != 0) continue;
        bool found = false;
        for (int32_t c : cand) if (c == s) { found = true; break; }
        if (!found) for (int32_t c : extra) if (c == s) { found = true; break; }
        index++;
        if (skip > 1 && index % skip != 0) continue;
        if (found) continue;
        if (ncand0 + (int)extra.size() >= LIST) break;
        extra.push_back(s);
    }
    int ne = (int)extra.size();
    std::vector<int> ex_depth(ne), ex_width(ne);
#pragma omp parallel for schedule(dynamic)
    for (int t = 0; t < ne; t++) {
        Levels lv = level_structure(g, extra[t]);
        ex_depth[t] = (int)lv.size();
        ex_width[t] = width_of(lv);
    }
    // pick max(depth - width), first wins (GPSOrder.cpp:614-624)
    int bestset = -1, bestval = -n;
    int32_t bestnode = start;
    for (int i = 0; i < ncand0 + ne; i++) {
        int eff = i < ncand0 ? cand_depth[i] - cand_width[i] : ex_depth[i - ncand0] - ex_width[i - ncand0];
        if (bestval < eff) { bestval = eff; bestset = i; bestnode = i < ncand0 ? cand[i] : extra[i - ncand0]; }
    }
    (void)bestset;
    Levels chosen = level_structure(g, bestnode);

    // number level by level (GPSOrder.cpp:394-450)
    Numbering num(g);
    {
        std::vector<Ranked> first;
        for (int32_t v : chosen[0]) first.push_back({v, num.nsum[v]});
        num.number_sorted(first);
        for (size_t j = 1; j < chosen.size(); j++) num.next_level(chosen[j - 1], chosen[j]);
    }
    if (num.cursor != n) throw std::runtime_error("gps_order: numbering incomplete");
    std::vector<int32_t> new_of = num.new_of;  // old -> new
    std::vector<int32_t> old_of = num.old_of;  // new -> old

    // in-block diagonal sort (GPSOrder.cpp:55-150): inside each full 64-row
    // block (except the last), if any of the first 32 diagonals is ~0, a
    // halving exchange pass moves larger diagonals forward.
    std::vector<double> dv(n, 0.0);
    std::vector<int32_t> ti(n);
    for (size_t k = 0; k < I.size(); k++)
        if (I[k] == J[k]) dv[new_of[I[k]]] = V[k];
    for (int i = 0; i < n; i++) ti[i] = i;
    const double tiny = 1e-8;
    for (int i = 0; i < n; i += 64) {
        if (i + 64 >= n) continue;
        int zc = 0;
        for (int j = 0; j < 32; j++)
            if (!(dv[i + j] > tiny || dv[i + j] < -tiny)) zc++;
        if (zc == 0) continue;
        for (int step = 32; step > 0; step /= 2)
            for (int j = 0; j < step; j++) {
                int k = i + j, m = i + j + step;
                if (dv[m] > dv[k]) { std::swap(dv[m], dv[k]); std::swap(ti[m], ti[k]); }
            }
    }
    ord.new_to_old.resize(n);
    ord.old_to_new.resize(n);
    for (int i = 0; i < n; i++) {
        ord.new_to_old[i] = old_of[ti[i]];
        ord.old_to_new[ord.new_to_old[i]] = i;
    }
    return ord;
}

}  // namespace sog
