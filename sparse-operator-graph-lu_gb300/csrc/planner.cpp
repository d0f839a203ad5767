// Recursive 2x2 block LU via explicit inverses, planned in two levels, then
// level-scheduled. Emits the same op DAG as the reference planner
// (BlockPlanner.cpp:103-374, 865-1292, 1305-1577; solver.cpp:56-110):
//
//   [L11,U11] = LU(A11); Li = L11^-1; Ui = U11^-1
//   U12 = Li*A12; L21 = A21*Ui; S = A22 - L21*U12; [L22,U22] = LU(S)
//
// Block matrices are quadtrees over a power-of-two grid of blocks; absent
// children are zero blocks and generate no ops.
#include <omp.h>
#include <parallel/algorithm>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <vector>

#include "plan.h"

namespace sog {
namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct QNode {
    int32_t level, id;
    int32_t ch[4];  // 0 = b11, 1 = b12, 2 = b21, 3 = b22; 0 = absent
};

// Append-only op list in fixed-size chunks: growing it never moves the ops
// already emitted (a 64^3 Laplacian emits 10.8M fine ops, 350 MB, which a
// doubling vector would copy and re-fault at every growth step).
struct OpLog {
    static constexpr int SHIFT = 18;  // 256K ops (8 MB) per chunk
    static constexpr int64_t MASK = (int64_t(1) << SHIFT) - 1;
    std::vector<std::unique_ptr<Op[]>> chunks;
    int64_t n = 0;
    void push_back(const Op& o) {
        if ((n >> SHIFT) == (int64_t)chunks.size()) chunks.emplace_back(new Op[size_t(1) << SHIFT]);
        chunks[n >> SHIFT][n & MASK] = o;
        n++;
    }
    int64_t size() const { return n; }
    Op& operator[](int64_t i) { return chunks[i >> SHIFT][i & MASK]; }
    const Op& operator[](int64_t i) const { return chunks[i >> SHIFT][i & MASK]; }
};

// Op emitter over one block-id space (one planning level).
struct Emitter {
    std::vector<QNode> nodes;  // nodes[0] is the "absent" sentinel
    OpLog ops;
    int32_t storage = 1;  // next block id; id 0 = none
    int32_t* seq;         // op sequence counter shared by both levels (operation.cpp:84-95)

    // node_hint: expected node count, reserved up front (untouched capacity
    // costs address space only)
    Emitter(int32_t* s, size_t node_hint) : seq(s) {
        nodes.reserve(node_hint);
        nodes.push_back({-1, 0, {0, 0, 0, 0}});
    }

    int32_t node(int level) {
        nodes.push_back({level, 0, {0, 0, 0, 0}});
        return (int32_t)nodes.size() - 1;
    }
    QNode& at(int32_t i) { return nodes[i]; }
    int32_t fresh_id() { return storage++; }
    void emit(int32_t op, int32_t src, int32_t src2, int32_t res, int32_t res2, int32_t group) {
        ops.push_back({op, src, src2, res, res2, 0, ++*seq, group});
    }
    int32_t child_or_new(int32_t c, int q) {
        int32_t k = at(c).ch[q];
        if (k == 0) {
            k = node(at(c).level - 1);
            at(c).ch[q] = k;
        }
        return k;
    }

    // c (+/-)= a * b  (BlockPlanner.cpp:1230-1283)
    void mul(int32_t a, int32_t b, int32_t c, int32_t group, int32_t kind) {
        if (a == 0 || b == 0) return;
        if (at(a).level == 0) {
            if (at(a).id > 0 && at(b).id > 0) {
                if (at(c).id <= 0) at(c).id = fresh_id();
                emit(kind, at(a).id, at(b).id, at(c).id, 0, group);
            }
            return;
        }
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 2; k++) {
                    int32_t ak = at(a).ch[i * 2 + k], bk = at(b).ch[k * 2 + j];
                    if (ak != 0 && bk != 0) {
                        int32_t ck = child_or_new(c, i * 2 + j);
                        mul(ak, bk, ck, group, kind);
                    }
                }
    }
    // c += a * b^T (BlockPlanner.cpp:1203-1229): quadrant (i, j) of c takes
    // a(i, k) * b(j, k)^T
    void mult(int32_t a, int32_t b, int32_t c, int32_t group) {
        if (a == 0 || b == 0) return;
        if (at(a).level == 0) {
            if (at(a).id > 0 && at(b).id > 0) {
                if (at(c).id <= 0) at(c).id = fresh_id();
                emit(OP_MULT, at(a).id, at(b).id, at(c).id, 0, group);
            }
            return;
        }
        for (int i = 0; i < 2; i++)
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 2; k++) {
                    int32_t ak = at(a).ch[i * 2 + k], bk = at(b).ch[j * 2 + k];
                    if (ak != 0 && bk != 0) {
                        int32_t ck = child_or_new(c, i * 2 + j);
                        mult(ak, bk, ck, group);
                    }
                }
    }
    // c = a - b, with copy / negate where one side is absent (BlockPlanner.cpp:1126-1201)
    void sub(int32_t a, int32_t b, int32_t c, int32_t group) {
        if (at(a).level == 0) {
            if (at(a).id > 0 || at(b).id > 0) {
                if (at(c).id <= 0) at(c).id = fresh_id();
                emit(OP_SUB, at(b).id, at(a).id, at(c).id, 0, group);
            }
            return;
        }
        for (int i = 0; i < 4; i++) {
            int32_t ai = at(a).ch[i], bi = at(b).ch[i];
            if (ai == 0 && bi == 0) continue;
            int32_t ci = child_or_new(c, i);
            if (ai != 0 && bi != 0) sub(ai, bi, ci, group);
            else if (ai != 0) copy(ai, ci, group);
            else neg(bi, ci, group);
        }
    }
    void copy(int32_t a, int32_t c, int32_t group) {
        if (at(a).level == 0) {
            if (at(a).id > 0) {
                if (at(c).id <= 0) at(c).id = fresh_id();
                emit(OP_SUB, 0, at(a).id, at(c).id, 0, group);
            }
            return;
        }
        for (int i = 0; i < 4; i++)
            if (at(a).ch[i] != 0) {
                int32_t ci = child_or_new(c, i);
                copy(at(a).ch[i], ci, group);
            }
    }
    void neg(int32_t b, int32_t c, int32_t group) {
        if (at(b).level == 0) {
            if (at(b).id > 0) {
                if (at(c).id <= 0) at(c).id = fresh_id();
                emit(OP_SUB, at(b).id, 0, at(c).id, 0, group);
            }
            return;
        }
        for (int i = 0; i < 4; i++)
            if (at(b).ch[i] != 0) {
                int32_t ci = child_or_new(c, i);
                neg(at(b).ch[i], ci, group);
            }
    }
    // y = l^-1 for block lower-triangular l; a3, when given, already holds the
    // inverse of l's leading quadrant (BlockPlanner.cpp:1019-1054).
    void inv_lower(int32_t l, int32_t y, int32_t a3, int32_t group) {
        if (at(l).level == 0) {
            if (at(l).id > 0) {
                at(y).id = fresh_id();
                emit(OP_LOWERINV, at(l).id, 0, at(y).id, 0, group);
            }
            return;
        }
        int32_t a = at(l).ch[0], c = at(l).ch[2], d = at(l).ch[3];
        int lev = at(a).level;
        int32_t d1 = node(lev);
        inv_lower(d, d1, 0, group);
        at(y).ch[3] = d1;
        int32_t d1c = node(lev);
        mul(d1, c, d1c, group, OP_MUL);
        int32_t a1 = a3;
        if (a1 == 0) {
            a1 = node(lev);
            inv_lower(a, a1, 0, group);
        }
        at(y).ch[0] = a1;
        int32_t c21 = node(lev);
        mul(d1c, a1, c21, group, OP_MULNEG);
        at(y).ch[2] = c21;
    }
    // y = u^-1 for block upper-triangular u (BlockPlanner.cpp:1056-1092).
    void inv_upper(int32_t u, int32_t y, int32_t a3, int32_t group) {
        if (at(u).level == 0) {
            if (at(u).id > 0) {
                at(y).id = fresh_id();
                emit(OP_UPPERINV, at(u).id, 0, at(y).id, 0, group);
            }
            return;
        }
        int32_t a = at(u).ch[0], b = at(u).ch[1], d = at(u).ch[3];
        int lev = at(a).level;
        int32_t a2 = a3;
        if (a2 == 0) {
            a2 = node(lev);
            inv_upper(a, a2, 0, group);
        }
        at(y).ch[0] = a2;
        int32_t a1b = node(lev);
        mul(a2, b, a1b, group, OP_MUL);
        int32_t d1 = node(lev);
        inv_upper(d, d1, 0, group);
        at(y).ch[3] = d1;
        int32_t a1bd1 = node(lev);
        mul(a1b, d1, a1bd1, group, OP_MULNEG);
        at(y).ch[1] = a1bd1;
    }
    // [l, u] = LU(a); l3/u3, when given, receive the inverses of l's and u's
    // leading quadrants for the caller to reuse (BlockPlanner.cpp:865-939).
    void lu(int32_t a, int32_t l, int32_t u, int32_t l3, int32_t u3, int32_t group) {
        if (at(a).level == 0) {
            if (at(a).id > 0) {
                if (at(l).id <= 0) at(l).id = fresh_id();
                if (at(u).id <= 0) at(u).id = fresh_id();
                emit(OP_LU, at(a).id, 0, at(l).id, at(u).id, group);
            }
            return;
        }
        int lev = at(a).level;
        int32_t ha = at(a).ch[0];
        int32_t l1 = node(lev - 1), u1 = node(lev - 1);
        int32_t l2 = l3, u2 = u3;
        if (l2 == 0) {
            l2 = node(lev - 1);
            u2 = node(lev - 1);
        }
        int32_t hl1 = 0, hu1 = 0;
        if (lev > 1) {
            hl1 = node(lev - 2);
            hu1 = node(lev - 2);
        }
        lu(ha, l1, u1, hl1, hu1, group);
        inv_lower(l1, l2, hl1, group);
        inv_upper(u1, u2, hu1, group);
        at(l).ch[0] = l1;
        at(u).ch[0] = u1;
        int32_t aua1b = node(lev - 1);
        int32_t b = at(a).ch[1];
        if (b != 0) {
            mul(l2, b, aua1b, group, OP_MUL);
            at(u).ch[1] = aua1b;
        }
        int32_t dsub = node(lev - 1);
        int32_t d = at(a).ch[3], c = at(a).ch[2];
        if (c != 0) {
            int32_t ca1al = node(lev - 1);
            mul(c, u2, ca1al, group, OP_MUL);
            at(l).ch[2] = ca1al;
            int32_t ca1b = node(lev - 1);
            mul(ca1al, aua1b, ca1b, group, OP_MUL);
            sub(d, ca1b, dsub, group);
        } else {
            dsub = d;
        }
        int32_t nl1 = node(lev - 1), nu1 = node(lev - 1);
        int32_t dl1 = 0, du1 = 0;
        if (lev > 1) {
            dl1 = node(lev - 2);
            du1 = node(lev - 2);
        }
        lu(dsub, nl1, nu1, dl1, du1, group);
        at(l).ch[3] = nl1;
        at(u).ch[3] = nu1;
    }

    // l = LL^T factor of symmetric a; l3, when given, receives the inverse of
    // l's leading quadrant (BlockPlanner.cpp:941-989):
    //   L11 = LLT(A11); Li = L11^-1; L21 = A21 Li^T; S = A22 - L21 L21^T; L22 = LLT(S)
    void llt(int32_t a, int32_t l, int32_t l3, int32_t group) {
        if (at(a).level == 0) {
            if (at(a).id > 0) {
                if (at(l).id <= 0) at(l).id = fresh_id();
                emit(OP_LLT, at(a).id, 0, at(l).id, 0, group);
            }
            return;
        }
        const int lev = at(a).level;
        int32_t ha = at(a).ch[0];
        int32_t l1 = node(lev - 1);
        int32_t l2 = l3 != 0 ? l3 : node(lev - 1);
        int32_t hl1 = lev > 1 ? node(lev - 2) : 0;
        llt(ha, l1, hl1, group);
        inv_lower(l1, l2, hl1, group);
        at(l).ch[0] = l1;
        int32_t dsub = node(lev - 1);
        int32_t d = at(a).ch[3], c = at(a).ch[2];
        if (c != 0) {
            int32_t ca1 = node(lev - 1), ca2 = node(lev - 1);
            mult(c, l2, ca1, group);
            at(l).ch[2] = ca1;
            mult(ca1, ca1, ca2, group);
            sub(d, ca2, dsub, group);
        } else {
            dsub = d;
        }
        int32_t nl1 = node(lev - 1);
        int32_t dl1 = lev > 1 ? node(lev - 2) : 0;
        llt(dsub, nl1, dl1, group);
        at(l).ch[3] = nl1;
    }

    // quadtree of input blocks over a grid of `rows` x `rows` blocks
    int32_t root_for(int rows) { return node(__builtin_popcount((unsigned)(rows - 1))); }
    // get-or-create the leaf at (bi, bj) (matrix.cpp:65-88); returns the leaf node
    int32_t leaf_at(int32_t root, int bi, int bj) {
        int32_t cur = root;
        for (int step = at(root).level; step > 0; step--) {
            int q = (((bi >> (step - 1)) & 1) << 1) | ((bj >> (step - 1)) & 1);
            cur = child_or_new(cur, q);
        }
        return cur;
    }
    int32_t find_leaf(int32_t root, int bi, int bj) {
        int32_t cur = root;
        for (int step = at(root).level; step > 0 && cur != 0; step--) {
            int q = (((bi >> (step - 1)) & 1) << 1) | ((bj >> (step - 1)) & 1);
            cur = at(cur).ch[q];
        }
        return cur;
    }
    void collect(int32_t m, int bi, int bj, std::vector<Leaf>& out) {
        if (m == 0) return;
        if (at(m).level == 0) {
            if (at(m).id > 0) out.push_back({bi, bj, at(m).id});
            return;
        }
        int h = 1 << (at(m).level - 1);
        for (int q = 0; q < 4; q++) collect(at(m).ch[q], bi + (q >> 1) * h, bj + (q & 1) * h, out);
    }
};

struct OpOrder {
    bool operator()(const Op& x, const Op& y) const {
        if (x.stage != y.stage) return x.stage < y.stage;
        if (x.group != y.group) return x.group < y.group;
        if (x.res != y.res) return x.res < y.res;
        if (x.src != y.src) return x.src < y.src;
        return x.seq < y.seq;
    }
};

// Liveness, dead-op elimination, stage assignment and ordering
// (BlockPlanner.cpp:103-374). `inputs` / `outputs` are block ids. The
// scheduled ops go to `out`, sorted by OpOrder; `log` gets its stages.
void schedule(OpLog& log, int32_t storage, const std::vector<int32_t>& inputs, const std::vector<int32_t>& outputs,
              bool always_prune, int threads, OpVec& out) {
    const int nthr = threads > 0 ? threads : omp_get_max_threads();
    const int64_t nops = log.size();
    std::vector<int32_t> lastuse(storage, 0), stage(storage, 0);
    stage[0] = 1;
    for (int32_t id : inputs) { stage[id] = 1; lastuse[id] = 0; }
    for (int32_t id : outputs) lastuse[id] = storage;
    // backward liveness: a source is live if any op writing a live block reads
    // it. Every reader of a block comes after its writers, so an op's results
    // have their final liveness when it is reached.
    for (int64_t i = nops - 1; i >= 0; i--) {
        const Op& o = log[i];
        int32_t mark = 0;
        if (o.res > 0) { mark = o.res; if (o.res2 > 0 && o.res2 > mark) mark = o.res2; }
        if (o.res > 0 && o.res2 > 0 && lastuse[o.res] == 0 && lastuse[o.res2] == 0) continue;
        if (o.res > 0 && o.res2 == 0 && lastuse[o.res] == 0) continue;
        if (mark > 0) {
            if (o.src > 0 && lastuse[o.src] < mark) lastuse[o.src] = mark;
            if (o.src2 > 0) {
                if (o.src2 >= storage) continue;
                if (lastuse[o.src2] < mark) lastuse[o.src2] = mark;
            }
        }
    }
    auto live = [&](const Op& o) { return lastuse[o.res] > 0 || (o.res2 > 0 && lastuse[o.res2] > 0); };
    // stage = 1 + max(stage of sources), at least 2 (BlockPlanner.cpp:225-266),
    // in op order. A dead op writes only dead blocks, which no live op reads,
    // so giving dead ops stages too leaves every live op's stage as it is when
    // the dead ones are removed first.
    int64_t waste = 0;
    for (int64_t i = 0; i < nops; i++) {
        Op& o = log[i];
        if (!live(o)) waste++;
        int32_t st = 0;
        if (o.src > 0) {
            st = std::max(stage[o.src] + 1, 2);
            if (o.src2 > 0) st = std::max(st, stage[o.src2] + 1);
        } else {
            if (o.src2 > 0) st = std::max(st, stage[o.src2] + 1);
            st = std::max(st, 2);
        }
        o.stage = st;
        if (o.res > 0 && stage[o.res] < st) stage[o.res] = st;
        if (o.res2 > 0 && stage[o.res2] < st) stage[o.res2] = st;
    }
    const bool prune = always_prune || waste > nops / 25;
    // kept ops, each single-result writer moved to its block's last write
    // stage, bucketed by stage: a counting sort over contiguous slices of the
    // log, one per thread (the order within a stage is fixed by the sort below)
    const int nslice = (int)std::max<int64_t>(1, std::min<int64_t>(nthr, nops / 65536 + 1));
    std::vector<int32_t> slice_max(nslice, 0);
    std::vector<std::vector<int64_t>> cnt(nslice);
    auto final_stage = [&](const Op& o) {
        return (o.res2 == 0 && o.res > 0 && stage[o.res] > o.stage) ? stage[o.res] : o.stage;
    };
    auto slice_lo = [&](int k) { return nops * k / nslice; };
#pragma omp parallel for schedule(static, 1) num_threads(nslice)
    for (int k = 0; k < nslice; k++) {
        int32_t mx = 0;
        for (int64_t i = slice_lo(k); i < slice_lo(k + 1); i++) {
            Op& o = log[i];
            o.stage = final_stage(o);
            mx = std::max(mx, o.stage);
        }
        slice_max[k] = mx;
    }
    int32_t maxst = 0;
    for (int32_t m : slice_max) maxst = std::max(maxst, m);
#pragma omp parallel for schedule(static, 1) num_threads(nslice)
    for (int k = 0; k < nslice; k++) {
        cnt[k].assign(maxst + 1, 0);
        for (int64_t i = slice_lo(k); i < slice_lo(k + 1); i++) {
            const Op& o = log[i];
            if (!prune || live(o)) cnt[k][o.stage]++;
        }
    }
    std::vector<int64_t> start(maxst + 2, 0);
    {
        int64_t run = 0;
        for (int32_t st = 0; st <= maxst; st++) {
            start[st] = run;
            for (int k = 0; k < nslice; k++) {
                const int64_t c = cnt[k][st];
                cnt[k][st] = run;  // slice k's first slot in stage st
                run += c;
            }
        }
        start[maxst + 1] = run;
    }
    out.resize(start[maxst + 1]);
#pragma omp parallel for schedule(static, 1) num_threads(nslice)
    for (int k = 0; k < nslice; k++)
        for (int64_t i = slice_lo(k); i < slice_lo(k + 1); i++) {
            const Op& o = log[i];
            if (!prune || live(o)) out[cnt[k][o.stage]++] = o;
        }
    // order each stage by OpOrder's remaining keys, stages in parallel: small
    // stages one per thread, large ones each with every thread. OpOrder is a
    // total order (seq is unique), so the result is the single sorted order.
    {
        constexpr int64_t BIG = 1 << 18;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthr)
        for (int32_t st = 0; st <= maxst; st++)
            if (start[st + 1] - start[st] < BIG)
                std::sort(out.begin() + start[st], out.begin() + start[st + 1], OpOrder());
        for (int32_t st = 0; st <= maxst; st++)
            if (start[st + 1] - start[st] >= BIG)
                __gnu_parallel::sort(out.begin() + start[st], out.begin() + start[st + 1], OpOrder(),
                                     __gnu_parallel::default_parallel_tag(nthr));
    }
    // stages of more than 8000 ops are split (BlockPlanner.cpp:335-354)
    int32_t jump = 0, band = 0, cur = 0;
    for (Op& o : out) {
        if (o.stage > cur) { cur = o.stage; band = 0; }
        if (band > 8000) { jump++; band = 0; }
        o.stage += jump;
        band++;
    }
}

}  // namespace

void mirror_triplets(int n, int64_t nnz, bool symmetric, const int32_t* I, const int32_t* J, const double* V,
                     std::vector<int32_t>& Io, std::vector<int32_t>& Jo, std::vector<double>& Vo) {
    Io.clear(); Jo.clear(); Vo.clear();
    Io.reserve(symmetric ? 2 * nnz : nnz);
    Jo.reserve(Io.capacity());
    Vo.reserve(Io.capacity());
    for (int64_t k = 0; k < nnz; k++) {
        if (I[k] < 0 || I[k] >= n || J[k] < 0 || J[k] >= n) throw std::runtime_error("triplet index out of range");
        Io.push_back(I[k]); Jo.push_back(J[k]); Vo.push_back(V ? V[k] : 0.0);
        if (symmetric && I[k] != J[k]) { Io.push_back(J[k]); Jo.push_back(I[k]); Vo.push_back(V ? V[k] : 0.0); }
    }
}

Plan build_plan(int n, int64_t nnz, bool symmetric, const int32_t* I0, const int32_t* J0, const double* V0,
                int threads) {
    if (n <= 0) throw std::runtime_error("dimension must be positive");
    Plan p;
    double t0 = now_s();
    std::vector<int32_t> I, J;
    std::vector<double> V;
    mirror_triplets(n, nnz, symmetric, I0, J0, V0, I, J, V);
    p.nval = nnz;
    if (symmetric) {
        p.mirror_src.reserve(I.size());
        for (int64_t k = 0; k < nnz; k++) {
            p.mirror_src.push_back((int32_t)k);
            if (I0[k] != J0[k]) p.mirror_src.push_back((int32_t)k);
        }
    }
    p.cfg = make_config(n);
    p.ord = gps_order(n, I, J, V, threads);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)I.size(); k++) { I[k] = p.ord.old_to_new[I[k]]; J[k] = p.ord.old_to_new[J[k]]; }
    p.t_order = now_s() - t0;
    double t1 = now_s();

    const int R = p.cfg.block_rows, R2 = p.cfg.block_rows_l2, bs2 = p.cfg.block_size_l2;
    const int sh2 = __builtin_popcount((unsigned)(bs2 - 1));
    const int n_ext = p.cfg.n_ext();
    int32_t seq = 0;

    // ---- coarse level (PlanL2, BlockPlanner.cpp:1470-1490): blocks in first-touch order
    Emitter cz(&seq, 1024);
    int32_t croot = cz.root_for(R2);
    std::vector<int32_t> cinputs;
    auto ctouch = [&](int bi, int bj) {
        int32_t lf = cz.leaf_at(croot, bi, bj);
        if (cz.at(lf).id == 0) { cz.at(lf).id = cz.fresh_id(); cinputs.push_back(cz.at(lf).id); }
        return lf;
    };
    for (size_t k = 0; k < I.size(); k++) ctouch(I[k] >> sh2, J[k] >> sh2);
    for (int i = n; i < n_ext; i++) ctouch(i / bs2, i / bs2);
    // symmetric input: the LL^T recursion (solver.cpp:70-71), L only
    p.symmetric = symmetric;
    int32_t cl = cz.root_for(R2), cu = cz.root_for(R2);
    if (symmetric) cz.llt(croot, cl, 0, 0);
    else cz.lu(croot, cl, cu, 0, 0, 0);
    p.coarse_ops_emitted = (int64_t)cz.ops.size();
    std::vector<Leaf> cL, cU;
    cz.collect(cl, 0, 0, cL);
    if (!symmetric) cz.collect(cu, 0, 0, cU);
    OpVec cops;
    {
        std::vector<int32_t> outs;
        for (auto& lf : cL) outs.push_back(lf.id);
        for (auto& lf : cU) outs.push_back(lf.id);
        schedule(cz.ops, cz.storage, cinputs, outs, true, threads, cops);
    }
    p.coarse_ops = (int64_t)cops.size();

    // ---- fine level: input tiles in (block row, block col) order (BlockPlanner.cpp:1491-1539)
    // a banded 64^3 Laplacian (R = 8192) creates ~260 fine nodes per block row
    Emitter fz(&seq, (size_t)512 * R + 1024);
    int32_t froot = fz.root_for(R);
    {
        std::vector<int64_t> keys(I.size());
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < (int64_t)I.size(); k++) keys[k] = (int64_t)(I[k] >> 6) * R + (J[k] >> 6);
        std::vector<int64_t> uk(keys);
        __gnu_parallel::sort(uk.begin(), uk.end(), std::less<int64_t>(),
                             __gnu_parallel::default_parallel_tag(threads > 0 ? threads : omp_get_max_threads()));
        uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
        for (int64_t key : uk) {
            int32_t lf = fz.leaf_at(froot, (int)(key / R), (int)(key % R));
            fz.at(lf).id = fz.fresh_id();
            p.input_bi.push_back((int32_t)(key / R));
            p.input_bj.push_back((int32_t)(key % R));
        }
        for (int i = n; i < n_ext; i++) {
            int bi = i >> 6;
            int32_t lf = fz.leaf_at(froot, bi, bi);
            if (fz.at(lf).id == 0) {
                fz.at(lf).id = fz.fresh_id();
                p.input_bi.push_back(bi);
                p.input_bj.push_back(bi);
            }
            p.pad_tile.push_back(fz.at(lf).id - 1);
            p.pad_off.push_back((int16_t)((i & 63) * 64 + (i & 63)));
        }
        p.n_input = fz.storage - 1;
        // the unpivoted recursion needs every diagonal block present (the
        // reference dereferences a missing one, BlockPlanner.cpp:881)
        for (int bi = 0; bi < R; bi++)
            if (fz.find_leaf(froot, bi, bi) == 0 || fz.at(fz.find_leaf(froot, bi, bi)).id == 0)
                throw std::runtime_error("structurally zero diagonal block " + std::to_string(bi));
        // value scatter: last occurrence of a duplicate wins
        p.scatter_tile.resize(I.size());
        p.scatter_off.resize(I.size());
        const int64_t nt = (int64_t)I.size();
        std::vector<std::pair<int64_t, int32_t>> slot(nt);  // (tile element, triplet): sorts stably by element
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < nt; k++) {
            const int32_t lf = fz.find_leaf(froot, I[k] >> 6, J[k] >> 6);  // read-only walk
            p.scatter_tile[k] = fz.nodes[lf].id - 1;
            p.scatter_off[k] = (int16_t)((I[k] & 63) * 64 + (J[k] & 63));
            slot[k] = {(int64_t)p.scatter_tile[k] * 4096 + p.scatter_off[k], (int32_t)k};
        }
        __gnu_parallel::sort(slot.begin(), slot.end(), std::less<std::pair<int64_t, int32_t>>(),
                             __gnu_parallel::default_parallel_tag(threads > 0 ? threads : omp_get_max_threads()));
        for (int64_t k = 0; k + 1 < nt; k++)
            if (slot[k].first == slot[k + 1].first) p.scatter_tile[slot[k].second] = -1;
    }
    std::vector<int32_t> finputs;
    for (int32_t id = 1; id <= p.n_input; id++) finputs.push_back(id);

    // coarse input block -> fine subtree at the same position (matrixZoomSet, BlockPlanner.cpp:1305-1315)
    const int scale = bs2 / 64;
    const int levL2 = __builtin_popcount((unsigned)(scale - 1));
    std::vector<int32_t> zoom(cz.storage, 0);
    {
        std::vector<Leaf> cin;
        cz.collect(croot, 0, 0, cin);
        for (auto& lf : cin) {
            int32_t cur = froot;
            int fl = fz.at(froot).level;
            int bi = lf.bi * scale, bj = lf.bj * scale;
            for (int step = fl; step > levL2 && cur != 0; step--) {
                int q = (((bi >> (step - 1)) & 1) << 1) | ((bj >> (step - 1)) & 1);
                cur = fz.at(cur).ch[q];
            }
            zoom[lf.id] = cur;
        }
    }
    // expand every coarse op into fine ops (copyOperatorL2, BlockPlanner.cpp:1332-1460)
    for (const Op& o : cops) {
        if (o.res > 0 && zoom[o.res] == 0) zoom[o.res] = fz.node(levL2);
        if (o.res2 > 0 && zoom[o.res2] == 0) zoom[o.res2] = fz.node(levL2);
        const int32_t g = o.seq;
        switch (o.op) {
            case OP_LOWERINV: fz.inv_lower(zoom[o.src], zoom[o.res], 0, g); break;
            case OP_UPPERINV: fz.inv_upper(zoom[o.src], zoom[o.res], 0, g); break;
            case OP_LU: fz.lu(zoom[o.src], zoom[o.res], zoom[o.res2], 0, 0, g); break;
            case OP_LLT: fz.llt(zoom[o.src], zoom[o.res], 0, g); break;
            case OP_MULT: fz.mult(zoom[o.src], zoom[o.src2], zoom[o.res], g); break;
            case OP_MUL: fz.mul(zoom[o.src], zoom[o.src2], zoom[o.res], g, OP_MUL); break;
            case OP_MULNEG: fz.mul(zoom[o.src], zoom[o.src2], zoom[o.res], g, OP_MULNEG); break;
            case OP_SUB:
                if (o.src > 0) {
                    if (o.src2 > 0) fz.sub(zoom[o.src2], zoom[o.src], zoom[o.res], g);
                    else fz.neg(zoom[o.src], zoom[o.res], g);
                } else if (o.src2 > 0) {
                    fz.copy(zoom[o.src2], zoom[o.res], g);
                }
                break;
            default: throw std::runtime_error("unexpected coarse op");
        }
    }
    p.fine_ops_emitted = (int64_t)fz.ops.size();
    // fine L/U leaves: coarse output leaves zoomed to their fine subtrees (matrixZoomUpdate)
    auto zoom_leaves = [&](const std::vector<Leaf>& cl_, std::vector<Leaf>& out) {
        for (auto& lf : cl_) {
            std::vector<Leaf> sub;
            fz.collect(zoom[lf.id], 0, 0, sub);
            for (auto& s : sub) out.push_back({lf.bi * scale + s.bi, lf.bj * scale + s.bj, s.id});
        }
        std::sort(out.begin(), out.end(), [](const Leaf& a, const Leaf& b) {
            return a.bi != b.bi ? a.bi < b.bi : a.bj < b.bj;
        });
    };
    zoom_leaves(cL, p.L);
    zoom_leaves(cU, p.U);
    {
        std::vector<int32_t> outs;
        for (auto& lf : p.L) outs.push_back(lf.id);
        for (auto& lf : p.U) outs.push_back(lf.id);
        schedule(fz.ops, fz.storage, finputs, outs, false, threads, p.ops);
    }
    p.storage_count = fz.storage;
    p.stages = p.ops.empty() ? 0 : p.ops.back().stage;
    p.t_plan = now_s() - t1;
    return p;
}

void scatter_tiles(const Plan& p, const double* V, double* tiles) {
    std::memset(tiles, 0, sizeof(double) * 4096 * (size_t)p.n_input);
    const bool mir = !p.mirror_src.empty();
    for (size_t k = 0; k < p.scatter_tile.size(); k++)
        if (p.scatter_tile[k] >= 0)
            tiles[(size_t)p.scatter_tile[k] * 4096 + p.scatter_off[k]] = V[mir ? p.mirror_src[k] : (int64_t)k];
    for (size_t k = 0; k < p.pad_tile.size(); k++) tiles[(size_t)p.pad_tile[k] * 4096 + p.pad_off[k]] = 1.0;
}

}  // namespace sog
