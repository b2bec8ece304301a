// Octree and U/V/W/X interaction lists of the reference's black-box FMM (host C++).
//
// Same tree as bbfmm::tree::populate (bbfmm.cpp:8-138):
//   root = anisotropic bounding box of the sources (getCenterRadius, bbfmm.cpp:43-65);
//   a node splits while nSource > maxPoint and level < maxLevel (bbfmm.cpp:81); all 8
//   children are created, child id = 4z + 2y + x with `coordinate < centre ? 0 : 1`;
//   child centre = c + (bit - 1/2) r, child radius = r / 2 (bbfmm.cpp:88-101).
// Same lists as tree::buildNode (bbfmm.cpp:158-241): the 6x6x6 same-level candidates around
// the parent, findNode (bbfmm.cpp:244-258) and isAdjacent (bbfmm.cpp:260-280).  Here nodes
// carry integer lattice coordinates, so findNode is a descent on coordinate bits and
// isAdjacent an interval test; the reference's EPS = 1e-12 tolerances only absorb rounding of
// the same lattice, so the lists are identical (checked against the reference's own trees).
//
// Points are kept in a stable per-node partition (the order the reference's sourceIndex
// vectors hold), so every node owns one contiguous range of the tree-ordered points.

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdlib>
#include <unordered_map>

#include <omp.h>

#include "internal.cuh"

namespace ibim {

namespace {

struct BNode {
    int level, parent, index8, leaf = 0, empty = 0;
    int child[8];
    double c[3], r[3];
    int coord[3];
    int sb, se, tb, te;  // ranges into the source / target permutations
};

struct Builder {
    const double *src, *tgt;
    bool same = false;  // targets are the sources: one partition serves both
    int maxpoint, maxlevel;
    std::vector<BNode> nodes;
    std::vector<int> *sp = nullptr, *tp = nullptr;
    std::vector<int> tmp;

    // assignChildren (bbfmm.cpp:67-138) for one node: leaf test, 8 children, partitions.
    // Returns false when the node stays a leaf.
    bool split_one(int id) {
        BNode &n0 = nodes[id];
        const int ns = n0.se - n0.sb;
        if (ns == 0) {
            n0.leaf = 1;
            n0.empty = 1;
            return false;
        }
        if (ns <= maxpoint || n0.level == maxlevel) {
            n0.leaf = 1;
            return false;
        }
        const int first = (int)nodes.size();
        for (int i = 0; i < 8; ++i) {
            BNode q;
            const BNode &p = nodes[id];
            q.level = p.level + 1;
            q.parent = id;
            q.index8 = i;
            for (int a = 0; a < 8; ++a) q.child[a] = -1;
            q.c[0] = p.c[0] + ((i & 1) - 0.5) * p.r[0];
            q.c[1] = p.c[1] + (((i >> 1) & 1) - 0.5) * p.r[1];
            q.c[2] = p.c[2] + ((i >> 2) - 0.5) * p.r[2];
            q.r[0] = p.r[0] * 0.5;
            q.r[1] = p.r[1] * 0.5;
            q.r[2] = p.r[2] * 0.5;
            q.coord[0] = 2 * p.coord[0] + (i & 1);
            q.coord[1] = 2 * p.coord[1] + ((i >> 1) & 1);
            q.coord[2] = 2 * p.coord[2] + (i >> 2);
            nodes.push_back(q);
        }
        for (int i = 0; i < 8; ++i) nodes[id].child[i] = first + i;
        partition(nodes[id], first, *sp, src, true);
        if (same) {
            for (int i = 0; i < 8; ++i) {
                nodes[first + i].tb = nodes[first + i].sb;
                nodes[first + i].te = nodes[first + i].se;
            }
        } else {
            partition(nodes[id], first, *tp, tgt, false);
        }
        return true;
    }
    void split(int id) {
        if (!split_one(id)) return;
        const int first = nodes[id].child[0];
        for (int i = 0; i < 8; ++i) split(first + i);
    }

    // stable 8-way partition of a node's range by octant; ranges of 16k points and more (the
    // top levels, built outside any parallel region) by all threads: per-thread octant counts
    // over contiguous slices, then each thread scatters its slice in order
    void partition(const BNode &p, int first, std::vector<int> &perm, const double *pts, bool is_src) {
        const int b = is_src ? p.sb : p.tb, e = is_src ? p.se : p.te;
        auto oct = [&](int idx) {
            const double *x = pts + 3 * (long)idx;
            return 4 * (x[2] < p.c[2] ? 0 : 1) + 2 * (x[1] < p.c[1] ? 0 : 1) + (x[0] < p.c[0] ? 0 : 1);
        };
        tmp.resize(std::max<size_t>(tmp.size(), (size_t)(e - b)));
        const int nthr = (e - b >= (1 << 14) && !omp_in_parallel()) ? std::min(64, omp_get_max_threads()) : 1;
        std::vector<std::array<int, 8>> cnt(nthr);
        std::vector<unsigned char> o8(nthr > 1 ? e - b : 0);
        auto slice = [&](int t, int &s0, int &s1) {
            s0 = b + (int)((long)(e - b) * t / nthr);
            s1 = b + (int)((long)(e - b) * (t + 1) / nthr);
        };
#pragma omp parallel for schedule(static) num_threads(nthr) if (nthr > 1)
        for (int t = 0; t < nthr; ++t) {
            int s0, s1;
            slice(t, s0, s1);
            std::array<int, 8> c{};
            for (int i = s0; i < s1; ++i) {
                const int o = oct(perm[i]);
                if (nthr > 1) o8[i - b] = (unsigned char)o;
                c[o]++;
            }
            cnt[t] = c;
        }
        // cnt[t][o] becomes thread t's first slot for octant o
        int o = b;
        for (int i = 0; i < 8; ++i) {
            BNode &q = nodes[first + i];
            const int start = o;
            for (int t = 0; t < nthr; ++t) {
                const int c = cnt[t][i];
                cnt[t][i] = o;
                o += c;
            }
            if (is_src) { q.sb = start; q.se = o; } else { q.tb = start; q.te = o; }
        }
#pragma omp parallel for schedule(static) num_threads(nthr) if (nthr > 1)
        for (int t = 0; t < nthr; ++t) {
            int s0, s1;
            slice(t, s0, s1);
            std::array<int, 8> &off = cnt[t];
            for (int i = s0; i < s1; ++i) tmp[off[nthr > 1 ? o8[i - b] : oct(perm[i])]++ - b] = perm[i];
        }
#pragma omp parallel for schedule(static) if (nthr > 1)
        for (int i = b; i < e; ++i) perm[i] = tmp[i - b];
    }
};

// The reference's node ids: creation order of its recursive assignChildren, which gives a
// node's 8 children consecutive ids when the node is split and then recurses into child 0..7.
void reference_ids(const std::vector<BNode> &nodes, std::vector<int> &ref) {
    ref.assign(nodes.size(), 0);
    int next = 1;
    std::vector<std::pair<int, int>> stack{{0, 0}};  // (node, next child to descend into)
    while (!stack.empty()) {
        auto &top = stack.back();
        const BNode &n = nodes[top.first];
        if (n.child[0] < 0) {
            stack.pop_back();
            continue;
        }
        if (top.second == 0) {
            for (int i = 0; i < 8; ++i) ref[n.child[i]] = next + i;
            next += 8;
        }
        if (top.second == 8) {
            stack.pop_back();
            continue;
        }
        const int c = n.child[top.second++];
        stack.push_back({c, 0});
    }
}

}  // namespace

TreeHost build_tree(const double *src, long ns, const double *tgt, long nt, int maxpoint, int maxlevel) {
    IBIM_REQUIRE(ns > 0, "FMM tree needs at least one source point");
    IBIM_REQUIRE(maxpoint > 0, "fmm_maxpoint must be positive");
    IBIM_REQUIRE(maxlevel >= 0 && maxlevel <= 18, "fmm_maxlevel must be in [0, 18]");
    Builder B;
    B.src = src;
    B.tgt = tgt;
    B.maxpoint = maxpoint;
    B.maxlevel = maxlevel;
    // getCenterRadius (bbfmm.cpp:43-65)
    double mx[3], mn[3];
    {
        double x0 = src[0], x1 = src[0], y0 = src[1], y1 = src[1], z0 = src[2], z1 = src[2];
#pragma omp parallel for schedule(static) reduction(min : x0, y0, z0) reduction(max : x1, y1, z1) if (ns >= (1 << 16))
        for (long i = 0; i < ns; ++i) {
            x0 = std::min(x0, src[3 * i]);
            x1 = std::max(x1, src[3 * i]);
            y0 = std::min(y0, src[3 * i + 1]);
            y1 = std::max(y1, src[3 * i + 1]);
            z0 = std::min(z0, src[3 * i + 2]);
            z1 = std::max(z1, src[3 * i + 2]);
        }
        mn[0] = x0, mn[1] = y0, mn[2] = z0;
        mx[0] = x1, mx[1] = y1, mx[2] = z1;
    }
    BNode root;
    root.level = 0;
    root.parent = -1;
    root.index8 = 0;
    for (int a = 0; a < 8; ++a) root.child[a] = -1;
    for (int a = 0; a < 3; ++a) {
        root.c[a] = (mx[a] + mn[a]) / 2.0;
        root.r[a] = (mx[a] - mn[a]) / 2.0;
        root.coord[a] = 0;
    }
    root.sb = 0;
    root.se = (int)ns;
    root.tb = 0;
    root.te = (int)nt;
    std::vector<int> sp(ns), tp;
    for (long i = 0; i < ns; ++i) sp[i] = (int)i;
    B.same = (tgt == src && nt == ns);
    if (!B.same) {
        tp.resize(nt);
        for (long i = 0; i < nt; ++i) tp[i] = (int)i;
    }
    B.sp = &sp;
    B.tp = B.same ? &sp : &tp;
    B.nodes.reserve(1024);
    B.nodes.push_back(root);
    // the top two levels serially, then the subtrees below them in parallel (disjoint point
    // ranges), each into its own node list, appended in subtree order
    std::vector<int> frontier{0};
    for (int l = 0; l < 2; ++l) {
        std::vector<int> next;
        for (int id : frontier)
            if (B.split_one(id))
                for (int i = 0; i < 8; ++i) next.push_back(B.nodes[id].child[i]);
        frontier.swap(next);
    }
    std::vector<Builder> sub(frontier.size());
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < (int)frontier.size(); ++k) {
        Builder &S = sub[k];
        S.src = B.src;
        S.tgt = B.tgt;
        S.same = B.same;
        S.maxpoint = B.maxpoint;
        S.maxlevel = B.maxlevel;
        S.sp = B.sp;
        S.tp = B.tp;
        S.nodes.push_back(B.nodes[frontier[k]]);
        S.nodes[0].parent = -1;
        S.split(0);
    }
    // subtree k's local node j >= 1 goes to base[k] + j (subtrees appended in order), in parallel
    std::vector<int> base(frontier.size() + 1);
    base[0] = (int)B.nodes.size() - 1;
    for (size_t k = 0; k < frontier.size(); ++k) base[k + 1] = base[k] + (int)sub[k].nodes.size() - 1;
    B.nodes.resize((size_t)base[frontier.size()] + 1);
#pragma omp parallel for schedule(dynamic, 1)
    for (int k = 0; k < (int)frontier.size(); ++k) {
        const int g = frontier[k], b = base[k];
        auto map = [&](int j) { return j == 0 ? g : b + j; };
        const std::vector<BNode> &L = sub[k].nodes;
        B.nodes[g].leaf = L[0].leaf;
        B.nodes[g].empty = L[0].empty;
        for (int i = 0; i < 8; ++i) B.nodes[g].child[i] = L[0].child[i] < 0 ? -1 : map(L[0].child[i]);
        for (size_t j = 1; j < L.size(); ++j) {
            BNode &q = B.nodes[(size_t)b + j];
            q = L[j];
            q.parent = map(q.parent);
            for (int i = 0; i < 8; ++i) q.child[i] = q.child[i] < 0 ? -1 : map(q.child[i]);
        }
    }

    const int nn = (int)B.nodes.size();
    int depth = 0;
    for (auto &n : B.nodes) depth = std::max(depth, n.level);
    trace_mark("tree: nodes");
    // findNode: the node at the candidate's level if it exists, else the leaf that contains it
    auto find_node = [&](int level, const int c[3]) {
        int id = 0;
        while (B.nodes[id].level < level && !B.nodes[id].leaf) {
            const int sh = level - B.nodes[id].level - 1;
            const int ch = ((c[2] >> sh) & 1) * 4 + ((c[1] >> sh) & 1) * 2 + ((c[0] >> sh) & 1);
            id = B.nodes[id].child[ch];
        }
        return id;
    };
    // isAdjacent: touching in one axis, overlapping or touching in the other two
    auto adjacent = [&](int a, int b) {
        const BNode &A = B.nodes[a], &Bn = B.nodes[b];
        bool touch[3], ot[3];
        for (int d = 0; d < 3; ++d) {
            const long la = (long)A.coord[d] << (depth - A.level), ha = (long)(A.coord[d] + 1) << (depth - A.level);
            const long lb = (long)Bn.coord[d] << (depth - Bn.level), hb = (long)(Bn.coord[d] + 1) << (depth - Bn.level);
            touch[d] = (ha == lb) || (hb == la);
            ot[d] = la <= hb && lb <= ha;
        }
        return (touch[0] && ot[1] && ot[2]) || (touch[1] && ot[0] && ot[2]) || (touch[2] && ot[0] && ot[1]);
    };
    // Lists are appended to per-thread buffers (one per list kind): a node is handled by one
    // thread, so its list is one contiguous segment [lbeg, lbeg + llen) of its thread's buffer
    // (no per-node allocations)
    const int nthr_l = omp_get_max_threads();
    std::vector<std::array<std::vector<int>, 4>> lbuf(nthr_l);
    std::vector<std::array<long, 4>> lbeg(nn);
    std::vector<std::array<int, 4>> llen(nn);
    std::vector<int> lown(nn, 0);
    for (auto &b4 : lbuf)
        for (auto &b : b4) b.reserve(1 << 16);
    // The candidates of a node are the 6 x 6 x 6 same-level cells around its parent, i.e. the
    // children of the parent's 3 x 3 x 3 neighbourhood: findNode is resolved once per parent
    // neighbour and shared by the 8 siblings.  A coarser leaf met by several candidates is
    // listed once (the reference's lists are sets).
    std::vector<int> parents;
    for (int id = 0; id < nn; ++id)
        if (B.nodes[id].child[0] >= 0) parents.push_back(id);
    enum { LU = 0, LV = 1, LW = 2, LX = 3 };
#pragma omp parallel for schedule(dynamic, 16)
    for (int k = 0; k < (int)parents.size(); ++k) {
        const int pid = parents[k];
        const BNode &pn = B.nodes[pid];
        const int pside = 1 << pn.level;
        int nb[27];
        for (int d = 0; d < 27; ++d) {
            const int c[3] = {pn.coord[0] + d % 3 - 1, pn.coord[1] + (d / 3) % 3 - 1, pn.coord[2] + d / 9 - 1};
            nb[d] = (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= pside || c[1] >= pside || c[2] >= pside)
                        ? -1
                        : find_node(pn.level, c);
        }
        std::vector<int> queue;
        std::array<std::vector<int>, 4> &buf = lbuf[omp_get_thread_num()];
        for (int ci = 0; ci < 8; ++ci) {
            const int id = pn.child[ci];
            const BNode &n = B.nodes[id];
            lown[id] = omp_get_thread_num();
            for (int w = 0; w < 4; ++w) lbeg[id][w] = (long)buf[w].size();
            auto push = [&](int w, int x) { buf[w].push_back(x); };
            // A candidate in a parent neighbour that is a leaf (at the parent's level or coarser)
            // is that leaf, shared by the neighbour's 8 cells and possibly by other neighbours:
            // it is classified once, at its first occurrence (the reference's lists are sets).
            int seen[27], nseen = 0;
            for (int xi = -2; xi < 4; ++xi)
                for (int yi = -2; yi < 4; ++yi)
                    for (int zi = -2; zi < 4; ++zi) {
                        const int m = nb[(xi >= 0 ? xi / 2 : -1) + 1 + 3 * ((yi >= 0 ? yi / 2 : -1) + 1) +
                                         9 * ((zi >= 0 ? zi / 2 : -1) + 1)];
                        if (m < 0) continue;
                        const int c[3] = {2 * pn.coord[0] + xi, 2 * pn.coord[1] + yi, 2 * pn.coord[2] + zi};
                        if (c[0] == n.coord[0] && c[1] == n.coord[1] && c[2] == n.coord[2]) continue;
                        const BNode &mn = B.nodes[m];
                        if (!(mn.level == pn.level && mn.child[0] >= 0)) {  // coarser than the child
                            bool dup = false;
                            for (int q = 0; q < nseen && !dup; ++q) dup = seen[q] == m;
                            if (dup) continue;
                            seen[nseen++] = m;
                            if (adjacent(id, m)) {
                                if (mn.leaf) push(LU, m);
                            } else {
                                push(LX, m);
                            }
                            continue;
                        }
                        const int cid = mn.child[((c[2] & 1) << 2) | ((c[1] & 1) << 1) | (c[0] & 1)];
                        // same level: adjacent when the lattice cells differ by at most one in
                        // every axis (they are distinct)
                        const bool adj = std::abs(c[0] - n.coord[0]) <= 1 && std::abs(c[1] - n.coord[1]) <= 1 &&
                                         std::abs(c[2] - n.coord[2]) <= 1;
                        {
                            if (!adj) {
                                push(LV, cid);
                            } else if (n.leaf) {
                                queue.clear();
                                queue.push_back(cid);
                                for (size_t q = 0; q < queue.size(); ++q) {
                                    const int f = queue[q];
                                    if (!adjacent(f, id)) {
                                        push(LW, f);
                                    } else if (B.nodes[f].leaf) {
                                        push(LU, f);
                                    } else {
                                        for (int ch = 0; ch < 8; ++ch) queue.push_back(B.nodes[f].child[ch]);
                                    }
                                }
                            }
                        }
                    }
            if (n.leaf) push(LU, id);
            for (int w = 0; w < 4; ++w) llen[id][w] = (int)((long)buf[w].size() - lbeg[id][w]);
        }
    }
    // the root (no parent): its own U entry when it is a leaf
    for (int w = 0; w < 4; ++w) {
        lbeg[0][w] = (long)lbuf[0][w].size();
        llen[0][w] = 0;
    }
    lown[0] = 0;
    if (B.nodes[0].leaf) {
        lbuf[0][LU].push_back(0);
        llen[0][LU] = 1;
    }
    trace_mark("tree: U V W X lists");
    std::vector<int> ref_of;
    reference_ids(B.nodes, ref_of);
    // level-ordered renumbering: by level, then by the reference's id (its creation order, a
    // permutation of 0 .. nn-1), as a counting sort by level over the nodes in reference order
    std::vector<int> by_ref(nn), order(nn), lstart(depth + 2, 0);
    for (int i = 0; i < nn; ++i) {
        by_ref[ref_of[i]] = i;
        lstart[B.nodes[i].level + 1]++;
    }
    for (int l = 0; l <= depth; ++l) lstart[l + 1] += lstart[l];
    for (int r = 0; r < nn; ++r) order[lstart[B.nodes[by_ref[r]].level]++] = by_ref[r];
    std::vector<int> newid(nn);
    for (int i = 0; i < nn; ++i) newid[order[i]] = i;

    TreeHost T;
    T.nnodes = nn;
    T.nlevels = depth + 1;
    T.level_begin.assign(T.nlevels + 1, 0);
    T.center.resize(3 * nn);
    T.radius.resize(3 * nn);
    T.coord.resize(3 * nn);
    T.parent.resize(nn);
    T.index8.resize(nn);
    T.leaf.resize(nn);
    T.empty.resize(nn);
    T.src_begin.resize(nn);
    T.src_end.resize(nn);
    T.tgt_begin.resize(nn);
    T.tgt_end.resize(nn);
    T.ref_id.resize(nn);
    // compressed lists in the level-ordered numbering: sizes, offsets, then a parallel fill
    NodeLists *dstl[4] = {&T.U, &T.V, &T.W, &T.X};
    for (int w = 0; w < 4; ++w) {
        NodeLists &L = *dstl[w];
        L.off.assign(nn + 1, 0);
        for (int i = 0; i < nn; ++i) L.off[i + 1] = L.off[i] + llen[order[i]][w];
        L.idx.resize(L.off[nn]);
    }
    for (int i = 0; i < nn; ++i) T.level_begin[B.nodes[order[i]].level + 1]++;
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < nn; ++i) {
        const BNode &n = B.nodes[order[i]];
        for (int a = 0; a < 3; ++a) {
            T.center[3 * i + a] = n.c[a];
            T.radius[3 * i + a] = n.r[a];
            T.coord[3 * i + a] = n.coord[a];
        }
        T.parent[i] = n.parent < 0 ? -1 : newid[n.parent];
        T.index8[i] = n.index8;
        T.leaf[i] = n.leaf;
        T.empty[i] = n.empty;
        T.src_begin[i] = n.sb;
        T.src_end[i] = n.se;
        T.tgt_begin[i] = n.tb;
        T.tgt_end[i] = n.te;
        T.ref_id[i] = ref_of[order[i]];
        const int o = order[i];
        for (int w = 0; w < 4; ++w) {
            const int *in = lbuf[lown[o]][w].data() + lbeg[o][w];
            int *out = dstl[w]->idx.data() + dstl[w]->off[i];
            for (int q = 0; q < llen[o][w]; ++q) out[q] = newid[in[q]];
        }
    }
    for (int l = 0; l < T.nlevels; ++l) T.level_begin[l + 1] += T.level_begin[l];
    T.tgt_perm = B.same ? sp : std::move(tp);
    T.src_perm = std::move(sp);
    return T;
}

}  // namespace ibim
