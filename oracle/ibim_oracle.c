/*
 * ORACLE — test infrastructure only (see ibim_oracle.h).
 *
 * Plain-C restatement of the reference's IBIM Poisson-Boltzmann path.  Every function
 * names the reference lines it follows.  It is the checker for the CUDA path and the CPU
 * baseline of the benchmark; it is pinned against the reference's own outputs
 * (the .npz fixtures in tests/golden, generated by tests/golden/make_golden.py).
 *
 * Reference files: levelset.cpp, bbfmm.h, bbfmm.cpp, gmres.cpp, electric.cpp, main.cpp.
 */
#include "ibim_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define ORC_EPS 1e-12 /* utils.h:40 */
#define SQR(x) ((x) * (x))

/* ======================================================================================
 * Level set (levelset.cpp)
 * ====================================================================================== */

typedef struct {
    int nx, ny, nz;
} dims_t;

static inline long cell(const dims_t *d, int i, int j, int k) { return ((long)i * d->ny + j) * d->nz + k; }

/* Grid::get clamps indices (levelset.cpp:28-33). */
static inline double gget(const double *g, const dims_t *d, int i, int j, int k) {
    i = i < 0 ? 0 : (i > d->nx - 1 ? d->nx - 1 : i);
    j = j < 0 ? 0 : (j > d->ny - 1 ? d->ny - 1 : j);
    k = k < 0 ? 0 : (k > d->nz - 1 ? d->nz - 1 : k);
    return g[cell(d, i, j, k)];
}

/* levelset::setGradient for one axis (levelset.cpp:330-388): WENO5 one-sided derivatives
 * from a 7-point window w[0..6] centred on w[3]. */
static inline void weno5(const double *w, double h, double *up, double *un) {
    const double EPS_LS = 1e-6;
    double a = w[1] - w[0], b = w[2] - w[1], c = w[3] - w[2], d = w[4] - w[3], e = w[5] - w[4], f = w[6] - w[5];
    double df = (-b + 7.0 * (c + d) - e) / 12.0;
    a = b - a;
    b = c - b;
    c = d - c;
    d = e - d;
    e = f - e;
    double is0 = 13.0 * SQR(e - d) + 3.0 * SQR(e - 3.0 * d);
    double is1 = 13.0 * SQR(d - c) + 3.0 * SQR(d + c);
    double is2 = 13.0 * SQR(c - b) + 3.0 * SQR(3.0 * c - b);
    double a0 = 1.0 / SQR(EPS_LS + is0), a1 = 6.0 / SQR(EPS_LS + is1), a2 = 3.0 / SQR(EPS_LS + is2);
    double w1 = 1.0 / (a0 + a1 + a2), w0 = a0 * w1, w2 = a2 * w1;
    *up = (df + w0 * (e - 2 * d + c) / 3.0 + (w2 - 0.5) * (d - 2.0 * c + b) / 6.0) / h;
    is0 = 13.0 * SQR(a - b) + 3.0 * SQR(a - 3.0 * b);
    is1 = 13.0 * SQR(b - c) + 3.0 * SQR(b + c);
    is2 = 13.0 * SQR(c - d) + 3.0 * SQR(3.0 * c - d);
    a0 = 1.0 / SQR(EPS_LS + is0);
    a1 = 6.0 / SQR(EPS_LS + is1);
    a2 = 3.0 / SQR(EPS_LS + is2);
    w1 = 1.0 / (a0 + a1 + a2);
    w0 = a0 * w1;
    w2 = a2 * w1;
    *un = (df - w0 * (a - 2 * b + c) / 3.0 - (w2 - 0.5) * (b - 2 * c + d) / 6.0) / h;
}

/* setWindow + 3x setGradient (levelset.cpp:309-323, :330-388): up[3] forward, un[3] backward. */
static inline void gradients(const double *g, const dims_t *dm, double h, int i, int j, int k, double up[3],
                             double un[3]) {
    double w[7];
    for (int l = 0; l < 7; ++l) w[l] = gget(g, dm, i - 3 + l, j, k);
    weno5(w, h, &up[0], &un[0]);
    for (int l = 0; l < 7; ++l) w[l] = gget(g, dm, i, j - 3 + l, k);
    weno5(w, h, &up[1], &un[1]);
    for (int l = 0; l < 7; ++l) w[l] = gget(g, dm, i, j, k - 3 + l);
    weno5(w, h, &up[2], &un[2]);
}

/* levelset::getNorm(Dun, Dup) (levelset.cpp:294-301): sqrt sum max(Dun+, (-Dup)+)^2. */
static inline double godunov(const double n[3], const double p[3]) {
    double v = 0.;
    for (int i = 0; i < 3; ++i) {
        double a = n[i] > 0. ? n[i] : 0.;
        double b = p[i] < 0. ? -p[i] : 0.;
        double m = a > b ? a : b;
        v += SQR(m);
    }
    return sqrt(v);
}

/* levelset::expand (levelset.cpp:91-109).  Cells outside the grid are skipped (the reference
 * writes them through the unclamped Grid::set; the fixtures keep every touched cell inside). */
void orc_expand(double *g, int nx, int ny, int nz, double lox, double loy, double loz, double h, int band,
                const double *centers, const double *radii, int natoms, double probe) {
    dims_t dm = {nx, ny, nz};
    for (int a = 0; a < natoms; ++a) {
        const double cx = centers[3 * a], cy = centers[3 * a + 1], cz = centers[3 * a + 2];
        const double R = radii[a] + probe;
        const int r = (int)(R / h) + band;
        const int icx = (int)((cx - lox) / h), icy = (int)((cy - loy) / h), icz = (int)((cz - loz) / h);
#pragma omp parallel for collapse(2) schedule(static)
        for (int ia = icx - r; ia <= icx + r; ++ia) {
            for (int ib = icy - r; ib <= icy + r; ++ib) {
                for (int ic = icz - r; ic <= icz + r; ++ic) {
                    if (ia < 0 || ib < 0 || ic < 0 || ia >= nx || ib >= ny || ic >= nz) continue;
                    const double px = lox + ia * h - cx, py = loy + ib * h - cy, pz = loz + ic * h - cz;
                    double dist = R - sqrt(px * px + py * py + pz * pz);
                    const double old = gget(g, &dm, ia, ib, ic);
                    g[cell(&dm, ia, ib, ic)] = dist > old ? dist : old;
                }
            }
        }
    }
}

/* levelset::evolve (levelset.cpp:111-187): TVD-RK3 of phi_t + vel |grad phi| = 0. */
void orc_evolve(double *g, int nx, int ny, int nz, double h, double final_t, double vel, double cfl) {
    dims_t dm = {nx, ny, nz};
    double dt = cfl * h / vel;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    const long n = (long)nx * ny * nz;
    double *u1 = (double *)malloc(sizeof(double) * n), *u2 = (double *)malloc(sizeof(double) * n);
    for (int s = 0; s < steps; ++s) {
        for (int stage = 0; stage < 3; ++stage) {
            const double *src = stage == 0 ? g : (stage == 1 ? u1 : u2);
#pragma omp parallel for collapse(2) schedule(static)
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny; ++j)
                    for (int k = 0; k < nz; ++k) {
                        double up[3], un[3];
                        gradients(src, &dm, h, i, j, k, up, un);
                        const long I = cell(&dm, i, j, k);
                        const double nrm = godunov(un, up);
                        if (stage == 0)
                            u1[I] = g[I] - dt * vel * nrm;
                        else if (stage == 1)
                            u2[I] = (3 * g[I] + u1[I] - dt * vel * nrm) / 4.0;
                        else
                            g[I] = (g[I] + 2 * (u2[I] - dt * vel * nrm)) / 3.0;
                    }
        }
    }
    free(u1);
    free(u2);
}

/* levelset::countGradient (levelset.cpp:398-432). */
long orc_count_gradient(const double *g, int nx, int ny, int nz, double h, double thickness, double thres,
                        double *accum_error, long *total) {
    dims_t dm = {nx, ny, nz};
    long bad = 0, tot = 0;
    double acc = 0.;
#pragma omp parallel for collapse(2) reduction(+ : bad, tot, acc) schedule(static)
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                if (fabs(g[cell(&dm, i, j, k)]) < thickness * h) {
                    tot++;
                    double up[3], un[3];
                    gradients(g, &dm, h, i, j, k, up, un);
                    const double nr = godunov(un, up);
                    if (fabs(nr - 1.0) > thres) bad++;
                    acc += fabs(nr - 1.0);
                }
            }
    if (accum_error) *accum_error = acc;
    if (total) *total = tot;
    return bad;
}

/* levelset::reinitialize (levelset.cpp:191-287). */
int orc_reinitialize(double *g, const double *phi0, int nx, int ny, int nz, double h, double final_t, double vel,
                     double cfl, int thickness, double thres) {
    dims_t dm = {nx, ny, nz};
    double dt = cfl * h / vel;
    const double eps = h * h;
    const int steps = (int)(final_t / dt) + 1;
    dt = final_t / (double)steps;
    const long n = (long)nx * ny * nz;
    double *u1 = (double *)malloc(sizeof(double) * n), *u2 = (double *)malloc(sizeof(double) * n);
    int step = 0;
    long bad = orc_count_gradient(g, nx, ny, nz, h, (double)thickness, thres, NULL, NULL);
    while (bad != 0 && step < steps) {
        step++;
        for (int stage = 0; stage < 3; ++stage) {
            const double *src = stage == 0 ? g : (stage == 1 ? u1 : u2);
#pragma omp parallel for collapse(2) schedule(static)
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny; ++j)
                    for (int k = 0; k < nz; ++k) {
                        double up[3], un[3];
                        gradients(src, &dm, h, i, j, k, up, un);
                        const long I = cell(&dm, i, j, k);
                        const double sign = phi0[I] / (sqrt(SQR(phi0[I]) + eps));
                        const double nd = sign > 0. ? godunov(un, up) : godunov(up, un);
                        if (stage == 0)
                            u1[I] = g[I] - dt * vel * sign * (nd - 1.0);
                        else if (stage == 1)
                            u2[I] = (3 * g[I] + u1[I] - dt * vel * sign * (nd - 1.0)) / 4.0;
                        else
                            g[I] = (g[I] + 2 * (u2[I] - dt * vel * sign * (nd - 1.0))) / 3.0;
                    }
        }
        bad = orc_count_gradient(g, nx, ny, nz, h, (double)thickness, thres, NULL, NULL);
    }
    free(u1);
    free(u2);
    return step;
}

/* main.cpp:45-60 with s = 1: expand, evolve inward by the probe, flip sign, reinit twice. */
void orc_levelset_build(double *g, int nx, int ny, int nz, double lox, double loy, double loz, double h, int band,
                        double init, const double *centers, const double *radii, int natoms, double probe,
                        double reinit_t, int thickness, double thres, int steps[2]) {
    const long n = (long)nx * ny * nz;
    for (long i = 0; i < n; ++i) g[i] = init;
    orc_expand(g, nx, ny, nz, lox, loy, loz, h, band, centers, radii, natoms, probe);
    orc_evolve(g, nx, ny, nz, h, probe, 1.0, 0.2);
    double *phi0 = (double *)malloc(sizeof(double) * n);
    for (long i = 0; i < n; ++i) {
        g[i] *= -1.0;
        phi0[i] = g[i];
    }
    steps[0] = orc_reinitialize(g, phi0, nx, ny, nz, h, reinit_t, 1.0, 0.5, thickness, thres);
    memcpy(phi0, g, sizeof(double) * n);
    steps[1] = orc_reinitialize(g, phi0, nx, ny, nz, h, reinit_t, 1.0, 0.5, thickness, thres);
    free(phi0);
}

/* Surface::Surface (levelset.cpp:437-586). */
long orc_surface(double *g, int nx, int ny, int nz, double lox, double loy, double loz, double h, int thickness,
                 double *out7, long cap, long *inclusion) {
    dims_t dm = {nx, ny, nz};
    const double tw = thickness * h;
    const long n = (long)nx * ny * nz;
    /* (a) flood fill from cell 0: a visited cell with g > -tw marks its 6 neighbours
     * (levelset.cpp:444-524).  The visited set is order-independent; BFS queue here. */
    unsigned char *vis = (unsigned char *)calloc(n, 1);
    long *queue = (long *)malloc(sizeof(long) * n);
    long qh = 0, qt = 0;
    queue[qt++] = 0;
    vis[0] = 1;
    const long syz = (long)ny * nz;
    while (qh < qt) {
        const long cur = queue[qh++];
        if (!(g[cur] > -tw)) continue;
        const int I = (int)(cur / syz), J = (int)(cur / nz - (long)I * ny), K = (int)(cur % nz);
        long nb[6];
        int cnt = 0;
        if (I + 1 <= nx - 1) nb[cnt++] = cur + syz;
        if (I - 1 >= 0) nb[cnt++] = cur - syz;
        if (J + 1 <= ny - 1) nb[cnt++] = cur + nz;
        if (J - 1 >= 0) nb[cnt++] = cur - nz;
        if (K + 1 <= nz - 1) nb[cnt++] = cur + 1;
        if (K - 1 >= 0) nb[cnt++] = cur - 1;
        for (int c = 0; c < cnt; ++c)
            if (!vis[nb[c]]) {
                vis[nb[c]] = 1;
                queue[qt++] = nb[c];
            }
    }
    free(queue);
    /* (b) unreached tube cells are cavities (levelset.cpp:529-537). */
    const double incl = -(tw + 1e-15);
    long ninc = 0;
    for (long id = 0; id < n; ++id)
        if (!vis[id] && fabs(g[id]) < tw) {
            g[id] = incl;
            ninc++;
        }
    free(vis);
    if (inclusion) *inclusion = ninc;
    /* (c) tube points in (i, j, k) order (levelset.cpp:540-583). */
    long np = 0;
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k) {
                const double dist = gget(g, &dm, i, j, k);
                if (!(fabs(dist) < tw)) continue;
                if (np < cap) {
                    double up[3], un[3], nrm[3];
                    gradients(g, &dm, h, i, j, k, up, un);
                    for (int a = 0; a < 3; ++a) nrm[a] = (un[a] + up[a]) * 0.5;
                    double *o = out7 + 7 * np;
                    o[0] = (lox + i * h) - nrm[0] * dist;
                    o[1] = (loy + j * h) - nrm[1] * dist;
                    o[2] = (loz + k * h) - nrm[2] * dist;
                    o[3] = nrm[0];
                    o[4] = nrm[1];
                    o[5] = nrm[2];
                    o[6] = 0.5 * (1.0 + cos(M_PI * dist / tw)) / tw;
                }
                np++;
            }
    return np;
}

/* ======================================================================================
 * Octree and interaction lists (bbfmm.cpp)
 * ====================================================================================== */

typedef struct {
    int *v;
    int n, cap;
} ivec;

static void iv_push(ivec *a, int x) {
    if (a->n == a->cap) {
        a->cap = a->cap ? 2 * a->cap : 16;
        a->v = (int *)realloc(a->v, sizeof(int) * a->cap);
    }
    a->v[a->n++] = x;
}

static int icmp(const void *a, const void *b) { return (*(const int *)a > *(const int *)b) - (*(const int *)a < *(const int *)b); }

static void iv_unique(ivec *a) {
    if (a->n < 2) return;
    qsort(a->v, a->n, sizeof(int), icmp);
    int m = 1;
    for (int i = 1; i < a->n; ++i)
        if (a->v[i] != a->v[m - 1]) a->v[m++] = a->v[i];
    a->n = m;
}

typedef struct {
    int level, parent, child[8], index8;
    int leaf, empty;
    int nsrc, ntgt;
    double c[3], r[3];
    ivec src, tgt;
    ivec L[4]; /* U V W X */
} onode;

struct orc_tree {
    onode *nd;
    int n, cap;
    const double *src, *tgt;
    int ns, nt, maxpoint, maxlevel, deepest;
};

static int new_node(orc_tree *t, int level, int index8) {
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 64;
        t->nd = (onode *)realloc(t->nd, sizeof(onode) * t->cap);
    }
    onode *q = &t->nd[t->n];
    memset(q, 0, sizeof(onode));
    q->level = level;
    q->index8 = index8;
    q->parent = -1;
    for (int i = 0; i < 8; ++i) q->child[i] = -1;
    return t->n++;
}

/* tree::assignChildren (bbfmm.cpp:67-138): split while nSource > maxPoint and level < maxLevel;
 * child id = 4 z + 2 y + x with `coordinate < centre ? 0 : 1`. */
static void assign_children(orc_tree *t, int id) {
    if (t->nd[id].nsrc == 0) {
        t->nd[id].leaf = 1;
        t->nd[id].empty = 1;
        return;
    }
    if (t->nd[id].nsrc <= t->maxpoint || t->nd[id].level == t->maxlevel) {
        t->nd[id].leaf = 1;
        if (t->deepest < t->nd[id].level) t->deepest = t->nd[id].level;
        return;
    }
    int kids[8];
    for (int i = 0; i < 8; ++i) {
        int c = new_node(t, t->nd[id].level + 1, i);
        onode *p = &t->nd[id], *q = &t->nd[c];
        kids[i] = c;
        p->child[i] = c;
        q->parent = id;
        q->c[0] = p->c[0] + ((i & 1) - 0.5) * p->r[0];
        q->c[1] = p->c[1] + (((i >> 1) & 1) - 0.5) * p->r[1];
        q->c[2] = p->c[2] + ((i >> 2) - 0.5) * p->r[2];
        q->r[0] = p->r[0] * 0.5;
        q->r[1] = p->r[1] * 0.5;
        q->r[2] = p->r[2] * 0.5;
    }
    onode *p = &t->nd[id];
    for (int i = 0; i < p->nsrc; ++i) {
        const int idx = p->src.v[i];
        const double *x = t->src + 3 * idx;
        const int cb = 4 * (x[2] < p->c[2] ? 0 : 1) + 2 * (x[1] < p->c[1] ? 0 : 1) + (x[0] < p->c[0] ? 0 : 1);
        onode *q = &t->nd[kids[cb]];
        iv_push(&q->src, idx);
        q->nsrc++;
    }
    for (int i = 0; i < p->ntgt; ++i) {
        const int idx = p->tgt.v[i];
        const double *x = t->tgt + 3 * idx;
        const int cb = 4 * (x[2] < p->c[2] ? 0 : 1) + 2 * (x[1] < p->c[1] ? 0 : 1) + (x[0] < p->c[0] ? 0 : 1);
        onode *q = &t->nd[kids[cb]];
        iv_push(&q->tgt, idx);
        q->ntgt++;
    }
    for (int i = 0; i < 8; ++i) assign_children(t, kids[i]);
}

static inline int pt_eq(const double *a, const double *b) {
    return fabs(a[0] - b[0]) < ORC_EPS && fabs(a[1] - b[1]) < ORC_EPS && fabs(a[2] - b[2]) < ORC_EPS;
}

/* tree::findNode (bbfmm.cpp:244-258). */
static int find_node(const orc_tree *t, const double *p) {
    int id = 0;
    for (;;) {
        const onode *n = &t->nd[id];
        if (pt_eq(n->c, p) || n->leaf) return id;
        const int x = n->c[0] > p[0] ? 0 : 1, y = n->c[1] > p[1] ? 0 : 1, z = n->c[2] > p[2] ? 0 : 1;
        id = n->child[4 * z + 2 * y + x];
    }
}

/* tree::isAdjacent (bbfmm.cpp:260-280). */
static int is_adjacent(const orc_tree *t, int a, int b) {
    const onode *A = &t->nd[a], *B = &t->nd[b];
    double df[3], rr[3];
    int rd[3];
    for (int i = 0; i < 3; ++i) {
        df[i] = fabs(A->c[i] - B->c[i]);
        rr[i] = fabs(A->r[i] + B->r[i]);
        rd[i] = rr[i] >= df[i] - ORC_EPS;
    }
    const int xa = (fabs(df[0] - rr[0]) < ORC_EPS) && (rd[1] && rd[2]);
    const int ya = (fabs(df[1] - rr[1]) < ORC_EPS) && (rd[0] && rd[2]);
    const int za = (fabs(df[2] - rr[2]) < ORC_EPS) && (rd[1] && rd[0]);
    return xa || ya || za;
}

/* tree::buildNode (bbfmm.cpp:158-241). */
static void build_node(orc_tree *t, int id, const double *minp, const double *maxp) {
    onode *n = &t->nd[id];
    if (n->parent != -1) {
        const onode *pn = &t->nd[n->parent];
        const double dx = n->r[0], dy = n->r[1], dz = n->r[2];
        const double xs = pn->c[0] - dx, ys = pn->c[1] - dy, zs = pn->c[2] - dz;
        int *queue = NULL;
        int qcap = 0;
        for (int xi = -2; xi < 4; ++xi)
            for (int yi = -2; yi < 4; ++yi)
                for (int zi = -2; zi < 4; ++zi) {
                    double cur[3] = {xs + 2 * xi * dx, ys + 2 * yi * dy, zs + 2 * zi * dz};
                    int inside = 1;
                    for (int a = 0; a < 3; ++a)
                        if (!(cur[a] <= maxp[a] + ORC_EPS && cur[a] >= minp[a] - ORC_EPS)) inside = 0;
                    if (!inside || pt_eq(cur, n->c)) continue;
                    const int cid = find_node(t, cur);
                    const int adj = is_adjacent(t, id, cid);
                    const onode *cn = &t->nd[cid];
                    if (cn->level < n->level) {
                        if (adj) {
                            if (cn->leaf) iv_push(&n->L[0], cid);
                        } else {
                            iv_push(&n->L[3], cid);
                        }
                    }
                    if (cn->level == n->level) {
                        if (!adj) {
                            iv_push(&n->L[1], cid);
                        } else if (n->leaf) {
                            int qh = 0, qt = 0;
                            if (qcap < 64) {
                                qcap = 64;
                                queue = (int *)realloc(queue, sizeof(int) * qcap);
                            }
                            queue[qt++] = cid;
                            while (qh < qt) {
                                const int f = queue[qh++];
                                const onode *fn = &t->nd[f];
                                if (!is_adjacent(t, f, id)) {
                                    iv_push(&n->L[2], f);
                                } else if (fn->leaf) {
                                    iv_push(&n->L[0], f);
                                } else {
                                    if (qt + 8 > qcap) {
                                        qcap = 2 * (qt + 8);
                                        queue = (int *)realloc(queue, sizeof(int) * qcap);
                                    }
                                    for (int c = 0; c < 8; ++c) queue[qt++] = fn->child[c];
                                }
                            }
                        }
                    }
                }
        free(queue);
    }
    if (n->leaf) iv_push(&n->L[0], id);
    for (int l = 0; l < 4; ++l) iv_unique(&n->L[l]);
}

/* tree::populate + getCenterRadius (bbfmm.cpp:8-65). */
orc_tree *orc_tree_build(const double *src, int ns, const double *tgt, int nt, int maxpoint, int maxlevel) {
    orc_tree *t = (orc_tree *)calloc(1, sizeof(orc_tree));
    t->src = src;
    t->tgt = tgt;
    t->ns = ns;
    t->nt = nt;
    t->maxpoint = maxpoint;
    t->maxlevel = maxlevel;
    double mx[3], mn[3];
    for (int a = 0; a < 3; ++a) mx[a] = mn[a] = src[a];
    for (int i = 0; i < ns; ++i)
        for (int a = 0; a < 3; ++a) {
            const double v = src[3 * i + a];
            if (v > mx[a]) mx[a] = v;
            if (v < mn[a]) mn[a] = v;
        }
    int root = new_node(t, 0, 0);
    onode *r = &t->nd[root];
    for (int a = 0; a < 3; ++a) {
        r->c[a] = (mx[a] + mn[a]) / 2.0;
        r->r[a] = (mx[a] - mn[a]) / 2.0;
    }
    r->nsrc = ns;
    r->ntgt = nt;
    for (int i = 0; i < ns; ++i) iv_push(&r->src, i);
    for (int i = 0; i < nt; ++i) iv_push(&t->nd[root].tgt, i);
    assign_children(t, root);
    double minp[3], maxp[3];
    for (int a = 0; a < 3; ++a) {
        minp[a] = t->nd[0].c[a] - t->nd[0].r[a];
        maxp[a] = t->nd[0].c[a] + t->nd[0].r[a];
    }
#pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < t->n; ++i) build_node(t, i, minp, maxp);
    return t;
}

void orc_tree_free(orc_tree *t) {
    if (!t) return;
    for (int i = 0; i < t->n; ++i) {
        free(t->nd[i].src.v);
        free(t->nd[i].tgt.v);
        for (int l = 0; l < 4; ++l) free(t->nd[i].L[l].v);
    }
    free(t->nd);
    free(t);
}

int orc_tree_nnodes(const orc_tree *t) { return t->n; }

void orc_tree_node(const orc_tree *t, int id, int *ints6, double *cr6) {
    const onode *n = &t->nd[id];
    ints6[0] = n->level;
    ints6[1] = n->parent;
    ints6[2] = n->leaf;
    ints6[3] = n->empty;
    ints6[4] = n->nsrc;
    ints6[5] = n->ntgt;
    for (int a = 0; a < 3; ++a) {
        cr6[a] = n->c[a];
        cr6[3 + a] = n->r[a];
    }
}

int orc_tree_list(const orc_tree *t, int id, int which, int *out, int cap) {
    const ivec *l = &t->nd[id].L[which];
    for (int i = 0; i < l->n && i < cap; ++i) out[i] = l->v[i];
    return l->n;
}

/* ======================================================================================
 * Kernels (electric.cpp:67-291).  d = source - target (bbfmm.h:439: eval(source, target)).
 * ====================================================================================== */

static const int K3F1[9] = {0, 1, 2, 0, 1, 2, 0, 1, 2};
static const int K3F2[9] = {0, 1, 2, 1, 2, 0, 1, 2, 0};

static inline double k2_inner(const orc_kparams *p) {
    if (p->kappa == 0.) return 0.;
    return (exp(-p->kappa * p->vr) - 1.0 + p->kappa * p->vr) / p->kappa / 2.0 / M_PI / p->vr / p->vr;
}

/* One of the 16 scalar kernels. */
static double kscalar(const orc_kparams *p, int id, const double dd[3]) {
    const double d = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
    const double r = sqrt(d);
    if (id == 3) {
        if (r < p->vr) return k2_inner(p);
        return (1.0 - exp(-p->kappa * r)) / 4.0 / M_PI / r;
    }
    if (r < p->vr) return 0.;
    if (id <= 2) return dd[id] * (p->dE / p->dI * exp(-p->kappa * r) * (p->kappa * r + 1) - 1.) / 4.0 / M_PI / r / d;
    if (id >= 13)
        return -dd[id - 13] * (p->dI / p->dE * exp(-p->kappa * r) * (p->kappa * r + 1) - 1.) / 4.0 / M_PI / r / d;
    const int k = id - 4;
    const double t = p->kappa * r;
    const double f = (exp(-t) * ((t + 3) * t + 3) - 3.0) * dd[K3F1[k]] * dd[K3F2[k]] / d / d / r;
    if (k < 3) return (1 - exp(-t) * (t + 1)) * 1.0 / d / r + f;
    return f;
}

/* Fused 4x4 block: rows F, Gx, Gy, Gz; columns phiX, phiY, phiZ, dphi (row-major b[4][4]). */
static void kfused(const orc_kparams *p, const double dd[3], double *b) {
    const double d = dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2];
    const double r = sqrt(d);
    if (r < p->vr) {
        memset(b, 0, sizeof(double) * 16);
        b[3] = -k2_inner(p);
        return;
    }
    const double t = p->kappa * r;
    const double e = exp(-t);
    const double r3 = r * d;
    const double c1 = (p->dE / p->dI * e * (t + 1) - 1.) / (4.0 * M_PI * r3);
    const double c4 = -(p->dI / p->dE * e * (t + 1) - 1.) / (4.0 * M_PI * r3);
    const double k2 = (1.0 - e) / (4.0 * M_PI * r);
    const double hd = (1 - e * (t + 1)) / r3;
    const double ho = (e * ((t + 3) * t + 3) - 3.0) / (d * r3);
    for (int a = 0; a < 3; ++a) {
        b[a] = dd[a] * c1;
        for (int c = 0; c < 3; ++c) b[4 * (a + 1) + c] = ho * dd[a] * dd[c] + (a == c ? hd : 0.);
        b[4 * (a + 1) + 3] = -dd[a] * c4;
    }
    b[3] = -k2;
}

/* ======================================================================================
 * Black-box Chebyshev FMM (bbfmm.h:200-624), generalised to an no x nd kernel block.
 * ====================================================================================== */

typedef struct {
    int p, R;
    double cheb[16];
    double tnode[16][16]; /* T_k(cheb_i) */
    double *R8;           /* 8 x R x R, R8[id][row * R + col] */
} cheb_t;

/* Chebyshev polynomials T_0..T_{p-1} at x (getStandardChebyPoly, bbfmm.h:280-303). */
static inline void cheb_poly(int p, double x, double *T) {
    T[0] = 1.0;
    if (p > 1) T[1] = x;
    for (int i = 2; i < p; ++i) T[i] = 2.0 * x * T[i - 1] - T[i - 2];
}

/* S_p(x, cheb_m) for m = 0..p-1: (-1 + 2 sum_k T_k(x) T_k(cheb_m)) / p (bbfmm.h:409-419). */
static inline void interp1(const cheb_t *c, double x, double *S) {
    double T[16];
    cheb_poly(c->p, x, T);
    for (int m = 0; m < c->p; ++m) {
        double s = 0.;
        for (int k = 0; k < c->p; ++k) s += T[k] * c->tnode[m][k];
        S[m] = (-1.0 + 2.0 * s) * (1.0 / c->p);
    }
}

/* initialize: nodes, polynomials and the 8 parent<->child operators (bbfmm.h:273-367). */
static void cheb_init(cheb_t *c, int p) {
    c->p = p;
    c->R = p * p * p;
    for (int i = 0; i < p; ++i) c->cheb[i] = -cos((i + 0.5) * M_PI / p);
    for (int i = 0; i < p; ++i) cheb_poly(p, c->cheb[i], c->tnode[i]);
    double S[2][16][16];
    for (int a = 0; a < 2 * p; ++a) {
        const double x = a < p ? 0.5 * c->cheb[a] - 0.5 : 0.5 * c->cheb[a - p] + 0.5;
        double row[16];
        interp1(c, x, row);
        for (int m = 0; m < p; ++m) S[a / p][a % p][m] = row[m];
    }
    const int R = c->R;
    c->R8 = (double *)malloc(sizeof(double) * 8 * R * R);
    for (int id = 0; id < 8; ++id) {
        const int b0 = id & 1, b1 = (id >> 1) & 1, b2 = (id >> 2) & 1;
        for (int i = 0; i < p; ++i)
            for (int j = 0; j < p; ++j)
                for (int k = 0; k < p; ++k)
                    for (int l = 0; l < p; ++l)
                        for (int m = 0; m < p; ++m)
                            for (int n = 0; n < p; ++n)
                                c->R8[(long)id * R * R + (i * p * p + j * p + k) * R + (l * p * p + m * p + n)] =
                                    S[b2][i][l] * S[b1][j][m] * S[b0][k][n];
    }
}

/* Leaf interpolation matrix rows (getTransferParentToChildren, bbfmm.h:392-433): for point x in
 * node (c, r): w[l p^2 + j p + i] = Sx[i] Sy[j] Sz[l]. */
static inline void leaf_weights(const cheb_t *c, const double *x, const double *ctr, const double *rad, double *w) {
    double S[3][16];
    for (int a = 0; a < 3; ++a) interp1(c, (x[a] - ctr[a]) / rad[a], S[a]);
    const int p = c->p;
    for (int l = 0; l < p; ++l)
        for (int j = 0; j < p; ++j)
            for (int i = 0; i < p; ++i) w[l * p * p + j * p + i] = S[0][i] * S[1][j] * S[2][l];
}

static inline void kblock(const orc_kparams *kp, int kernel, const double dd[3], double *b) {
    if (kernel == ORC_KERNEL_FUSED)
        kfused(kp, dd, b);
    else
        b[0] = kscalar(kp, kernel, dd);
}

static void fmm_impl(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out,
                     const unsigned char *need);

void orc_fmm(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out) {
    fmm_impl(t, p, kp, kernel, dens, out, NULL);
}

/* Timing sample: the upward pass in full, the downward pass (M2L, L2L, near field, L2P) only
 * for nodes whose id is a multiple of `stride`; `out` is then incomplete. */
void orc_fmm_sample(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out,
                    int stride) {
    if (stride < 1) stride = 1;
    unsigned char *need = (unsigned char *)malloc((size_t)t->n);
    for (int i = 0; i < t->n; ++i) need[i] = i % stride == 0;
    fmm_impl(t, p, kp, kernel, dens, out, need);
    free(need);
}

/* The FMM at chosen targets only (a checker for large trees): the upward pass in full, the
 * downward pass for the leaves that hold the targets sel[0..nsel) and for their ancestors (whose
 * locals the leaves' L2L chain needs), in the same arithmetic order as orc_fmm, so out equals
 * orc_fmm's at those targets; elsewhere out is incomplete.  Returns the number of leaves. */
int orc_fmm_targets(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out,
                    const int *sel, int nsel) {
    int *leaf_of = (int *)malloc(sizeof(int) * (size_t)(t->nt > 0 ? t->nt : 1));
    for (int i = 0; i < t->nt; ++i) leaf_of[i] = -1;
    for (int i = 0; i < t->n; ++i)
        if (t->nd[i].leaf)
            for (int q = 0; q < t->nd[i].ntgt; ++q) leaf_of[t->nd[i].tgt.v[q]] = i;
    unsigned char *need = (unsigned char *)calloc((size_t)t->n, 1);
    int nleaf = 0;
    for (int q = 0; q < nsel; ++q) {
        if (sel[q] < 0 || sel[q] >= t->nt || leaf_of[sel[q]] < 0) continue;
        int i = leaf_of[sel[q]];
        if (!need[i]) ++nleaf;
        for (; i >= 0 && !need[i]; i = t->nd[i].parent) need[i] = 1;
    }
    fmm_impl(t, p, kp, kernel, dens, out, need);
    free(need);
    free(leaf_of);
    return nleaf;
}

static void fmm_impl(const orc_tree *t, int p, const orc_kparams *kp, int kernel, const double *dens, double *out,
                     const unsigned char *need) {
    const int nd = kernel == ORC_KERNEL_FUSED ? 4 : 1, no = nd, nb = nd * no;
    cheb_t ch;
    cheb_init(&ch, p);
    const int R = ch.R, nn = t->n;
    double *charge = (double *)calloc((size_t)nn * nd * R, sizeof(double));
    double *local = (double *)calloc((size_t)nn * no * R, sizeof(double));
    memset(out, 0, sizeof(double) * (size_t)no * t->nt);
    /* node Chebyshev points per axis (getScaledChebyNode, bbfmm.h:370-377) */
    double *cn = (double *)malloc(sizeof(double) * nn * 3 * p);
    for (int i = 0; i < nn; ++i)
        for (int a = 0; a < 3; ++a)
            for (int m = 0; m < p; ++m) cn[(i * 3 + a) * p + m] = t->nd[i].c[a] + t->nd[i].r[a] * ch.cheb[m];
    int maxl = 0;
    for (int i = 0; i < nn; ++i)
        if (t->nd[i].level > maxl) maxl = t->nd[i].level;
    /* upPass (bbfmm.h:500-536): leaf P2M, then M2M bottom-up. */
#pragma omp parallel for schedule(dynamic, 8)
    for (int i = 0; i < nn; ++i) {
        const onode *n = &t->nd[i];
        if (!n->leaf || n->empty) continue;
        double *w = (double *)malloc(sizeof(double) * R);
        for (int s = 0; s < n->nsrc; ++s) {
            const int idx = n->src.v[s];
            leaf_weights(&ch, t->src + 3 * idx, n->c, n->r, w);
            for (int d = 0; d < nd; ++d) {
                const double q = dens[(size_t)d * t->ns + idx];
                double *M = charge + ((size_t)i * nd + d) * R;
                for (int c = 0; c < R; ++c) M[c] += w[c] * q;
            }
        }
        free(w);
    }
    for (int lv = maxl - 1; lv >= 0; --lv) {
#pragma omp parallel for schedule(dynamic, 8)
        for (int i = 0; i < nn; ++i) {
            const onode *n = &t->nd[i];
            if (n->level != lv || n->leaf) continue;
            for (int c8 = 0; c8 < 8; ++c8) {
                const int ci = n->child[c8];
                if (t->nd[ci].empty) continue;
                const double *Rm = ch.R8 + (size_t)c8 * R * R;
                for (int d = 0; d < nd; ++d) {
                    const double *cm = charge + ((size_t)ci * nd + d) * R;
                    double *pm = charge + ((size_t)i * nd + d) * R;
                    for (int col = 0; col < R; ++col) {
                        double s = 0.;
                        for (int row = 0; row < R; ++row) s += Rm[row * R + col] * cm[row];
                        pm[col] += s;
                    }
                }
            }
        }
    }
    /* downPass (bbfmm.h:538-623): per level, V and X list M2L with the kernel evaluated at
     * Chebyshev node pairs, then L2L from the parent. */
    for (int lv = 1; lv <= maxl; ++lv) {
#pragma omp parallel for schedule(dynamic, 1)
        for (int i = 0; i < nn; ++i) {
            const onode *n = &t->nd[i];
            if (n->level != lv || (need && !need[i])) continue;
            double *L = local + (size_t)i * no * R;
            double blk[16];
            for (int which = 1; which <= 3; which += 2) {
                const ivec *lst = &n->L[which];
                for (int e = 0; e < lst->n; ++e) {
                    const int s = lst->v[e];
                    if (t->nd[s].empty) continue;
                    const double *scn = cn + (size_t)s * 3 * p, *tcn = cn + (size_t)i * 3 * p;
                    const double *M = charge + (size_t)s * nd * R;
                    for (int kt = 0; kt < p; ++kt)
                        for (int jt = 0; jt < p; ++jt)
                            for (int it = 0; it < p; ++it) {
                                const int ct = kt * p * p + jt * p + it;
                                double acc[4] = {0, 0, 0, 0};
                                for (int ks = 0; ks < p; ++ks)
                                    for (int js = 0; js < p; ++js)
                                        for (int is = 0; is < p; ++is) {
                                            const int cs = ks * p * p + js * p + is;
                                            const double dd[3] = {scn[is] - tcn[it], scn[p + js] - tcn[p + jt],
                                                                  scn[2 * p + ks] - tcn[2 * p + kt]};
                                            kblock(kp, kernel, dd, blk);
                                            for (int o = 0; o < no; ++o)
                                                for (int d = 0; d < nd; ++d)
                                                    acc[o] += blk[o * nd + d] * M[(size_t)d * R + cs];
                                        }
                                for (int o = 0; o < no; ++o) L[(size_t)o * R + ct] += acc[o];
                            }
                }
            }
            const double *Rm = ch.R8 + (size_t)n->index8 * R * R;
            const double *PL = local + (size_t)n->parent * no * R;
            for (int o = 0; o < no; ++o)
                for (int row = 0; row < R; ++row) {
                    double s = 0.;
                    for (int col = 0; col < R; ++col) s += Rm[row * R + col] * PL[(size_t)o * R + col];
                    L[(size_t)o * R + row] += s;
                }
        }
    }
    /* leaves: U and W lists direct, then L2P (bbfmm.h:571-610) */
    (void)nb;
#pragma omp parallel for schedule(dynamic, 1)
    for (int i = 0; i < nn; ++i) {
        const onode *n = &t->nd[i];
        if (!n->leaf || n->ntgt == 0 || (need && !need[i])) continue;
        double *w = (double *)malloc(sizeof(double) * R);
        double blk[16];
        for (int tt = 0; tt < n->ntgt; ++tt) {
            const int ti = n->tgt.v[tt];
            const double *x = t->tgt + 3 * ti;
            double acc[4] = {0, 0, 0, 0};
            for (int which = 0; which <= 2; which += 2) {
                const ivec *lst = &n->L[which];
                for (int e = 0; e < lst->n; ++e) {
                    const onode *sn = &t->nd[lst->v[e]];
                    if (sn->empty) continue;
                    for (int ss = 0; ss < sn->nsrc; ++ss) {
                        const int si = sn->src.v[ss];
                        const double *y = t->src + 3 * si;
                        const double dd[3] = {y[0] - x[0], y[1] - x[1], y[2] - x[2]};
                        kblock(kp, kernel, dd, blk);
                        for (int o = 0; o < no; ++o)
                            for (int d = 0; d < nd; ++d) acc[o] += blk[o * nd + d] * dens[(size_t)d * t->ns + si];
                    }
                }
            }
            leaf_weights(&ch, x, n->c, n->r, w);
            const double *L = local + (size_t)i * no * R;
            for (int o = 0; o < no; ++o) {
                double s = 0.;
                for (int c = 0; c < R; ++c) s += w[c] * L[(size_t)o * R + c];
                out[(size_t)o * t->nt + ti] += acc[o] + s;
            }
        }
        free(w);
    }
    free(cn);
    free(charge);
    free(local);
    free(ch.R8);
}

/* ======================================================================================
 * BIE operator, right-hand side, GMRES and energy (electric.cpp, gmres.cpp)
 * ====================================================================================== */

typedef struct {
    const double *surf7;
    long N;
    double h;
    const orc_bie_params *bp;
    orc_kparams kp;
    double *pts, *nrm, *w; /* SoA-ish copies: pts (N x 3), nrm (N x 3), w = weight * h^3 */
    orc_tree *tree;        /* mode 0 only */
} bie_t;

static void bie_init(bie_t *B, const double *surf7, long N, double h, const orc_bie_params *bp) {
    B->surf7 = surf7;
    B->N = N;
    B->h = h;
    B->bp = bp;
    B->kp.kappa = bp->kappa;
    B->kp.dE = bp->dE;
    B->kp.dI = bp->dI;
    B->kp.vr = bp->tau * h;
    B->pts = (double *)malloc(sizeof(double) * 3 * N);
    B->nrm = (double *)malloc(sizeof(double) * 3 * N);
    B->w = (double *)malloc(sizeof(double) * N);
    for (long i = 0; i < N; ++i) {
        for (int a = 0; a < 3; ++a) {
            B->pts[3 * i + a] = surf7[7 * i + a];
            B->nrm[3 * i + a] = surf7[7 * i + 3 + a];
        }
        B->w[i] = surf7[7 * i + 6] * 1.0 * h * SQR(h); /* electric.cpp:33 */
    }
    B->tree = bp->mode == 0 ? orc_tree_build(B->pts, (int)N, B->pts, (int)N, bp->maxpoint, bp->maxlevel) : NULL;
}

static void bie_free(bie_t *B) {
    orc_tree_free(B->tree);
    free(B->pts);
    free(B->nrm);
    free(B->w);
}

/* the four weighted densities of electric.cpp:321-329 (rows phiX, phiY, phiZ, dphi) */
static void bie_densities(const bie_t *B, const double *x, double *dens) {
    const long N = B->N;
    for (long i = 0; i < N; ++i) {
        dens[3 * N + i] = x[i + N] * B->w[i];
        for (int a = 0; a < 3; ++a) dens[a * N + i] = x[i] * B->nrm[3 * i + a] * B->w[i];
    }
}

static const int KDENS[16] = {0, 1, 2, 3, 0, 1, 2, 0, 1, 2, 1, 2, 0, 3, 3, 3};

/* dmapping (electric.cpp:294-388). */
static void bie_apply(void *ctx, const double *x, double *y) {
    bie_t *B = (bie_t *)ctx;
    const long N = B->N;
    const orc_bie_params *bp = B->bp;
    double *dens = (double *)malloc(sizeof(double) * 4 * N);
    bie_densities(B, x, dens);
    const double e1 = 0.5 * (1 + bp->dE / bp->dI), e2 = 0.5 * (1 + bp->dI / bp->dE);
    if (bp->mode == 0) {
        double *o = (double *)malloc(sizeof(double) * 4 * N);
        orc_fmm(B->tree, bp->np, &B->kp, ORC_KERNEL_FUSED, dens, o);
        for (long i = 0; i < N; ++i) {
            const double ng = B->nrm[3 * i] * o[N + i] + B->nrm[3 * i + 1] * o[2 * N + i] + B->nrm[3 * i + 2] * o[3 * N + i];
            y[i] = x[i] + o[i] / e1;
            y[i + N] = x[i + N] + ng / e2;
        }
        free(o);
    } else {
        double *r = (double *)malloc(sizeof(double) * 16 * N);
        for (int k = 0; k < 16; ++k) {
            orc_tree *t = orc_tree_build(B->pts, (int)N, B->pts, (int)N, bp->maxpoint, bp->maxlevel);
            orc_fmm(t, bp->np, &B->kp, k, dens + (size_t)KDENS[k] * N, r + (size_t)k * N);
            orc_tree_free(t);
        }
#define RK(k) r[(size_t)(k) * N + i]
        for (long i = 0; i < N; ++i) {
            const double nx = B->nrm[3 * i], ny = B->nrm[3 * i + 1], nz = B->nrm[3 * i + 2];
            const double t1 = nx * (RK(4) + RK(10) + RK(9)) + ny * (RK(5) + RK(7) + RK(11)) + nz * (RK(6) + RK(12) + RK(8));
            const double t2 = nx * RK(13) + ny * RK(14) + nz * RK(15);
            y[i] = x[i] + (RK(0) + RK(1) + RK(2) - RK(3)) / e1;
            y[i + N] = x[i + N] + (t1 - t2) / e2;
        }
#undef RK
        free(r);
    }
    free(dens);
}

void orc_matvec(const double *surf7, long N, double h, const orc_bie_params *bp, const double *x, double *y) {
    bie_t B;
    bie_init(&B, surf7, N, h, bp);
    bie_apply(&B, x, y);
    bie_free(&B);
}

void orc_rhs(const double *surf7, long N, const double *centers, const double *charges, int M,
             const orc_bie_params *bp, double *b) {
    const double e1 = 0.5 * (1 + bp->dE / bp->dI), e2 = 0.5 * (1 + bp->dI / bp->dE);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < N; ++i) {
        const double *s = surf7 + 7 * i;
        double b1 = 0., b2 = 0.;
        for (int a = 0; a < M; ++a) {
            const double dx = s[0] - centers[3 * a], dy = s[1] - centers[3 * a + 1], dz = s[2] - centers[3 * a + 2];
            const double d = dx * dx + dy * dy + dz * dz, r = sqrt(d);
            b1 += charges[a] / bp->dI / 4.0 / M_PI / r / e1;
            b2 -= charges[a] / bp->dI / 4.0 / M_PI / d / r * (s[3] * dx + s[4] * dy + s[5] * dz) / e2;
        }
        b[i] = b1;
        b[i + N] = b2;
    }
}

static double dot(long n, const double *a, const double *b) {
    double s = 0.;
    for (long i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* gmres.cpp:23-43 */
static void gen_rot(double dx, double dy, double *cs, double *sn) {
    if (dy == 0.0) {
        *cs = 1.0;
        *sn = 0.0;
    } else if (fabs(dy) > fabs(dx)) {
        const double t = dx / dy;
        *sn = 1.0 / sqrt(1.0 + t * t);
        *cs = t * *sn;
    } else {
        const double t = dy / dx;
        *cs = 1.0 / sqrt(1.0 + t * t);
        *sn = t * *cs;
    }
}

static void apply_rot(double *dx, double *dy, double cs, double sn) {
    const double t = cs * *dx + sn * *dy;
    *dy = -sn * *dx + cs * *dy;
    *dx = t;
}

/* gmres.cpp:9-21 (Update): back substitution on the rotated Hessenberg, x += V y. */
static void gm_update(long n, double *x, int k, const double *H, int ld, const double *s, double *const *v) {
    double y[256];
    for (int i = 0; i <= k; ++i) y[i] = s[i];
    for (int i = k; i >= 0; --i) {
        y[i] /= H[i * ld + i];
        for (int j = i - 1; j >= 0; --j) y[j] -= H[j * ld + i] * y[i];
    }
    for (int j = 0; j <= k; ++j)
        for (long q = 0; q < n; ++q) x[q] += y[j] * v[j][q];
}

/* GMRES (gmres.cpp:50-164): restarted, modified Gram-Schmidt, Givens rotations. */
int orc_gmres(orc_op A, void *ctx, long n, double *x, const double *b, int m, int max_iter, double tol, int *iters,
              int *matvecs) {
    if (m > 255) m = 255;
    int nmv = 0, j = 1, i = 0;
    double *r = (double *)malloc(sizeof(double) * n), *w = (double *)malloc(sizeof(double) * n);
    double s[256], cs[256], sn[256];
    double normb = sqrt(dot(n, b, b));
    A(ctx, x, w);
    nmv++;
    for (long q = 0; q < n; ++q) r[q] = b[q] - w[q];
    double beta = sqrt(dot(n, r, r)), resid;
    if (normb == 0.0) normb = 1;
    if ((resid = beta / normb) <= tol) {
        free(r);
        free(w);
        if (iters) *iters = 0;
        if (matvecs) *matvecs = nmv;
        return 0;
    }
    const int ld = m + 1;
    double *H = (double *)calloc((size_t)ld * ld, sizeof(double));
    double **v = (double **)malloc(sizeof(double *) * (m + 1));
    for (int k = 0; k <= m; ++k) v[k] = (double *)malloc(sizeof(double) * n);
    int rc = 1;
    while (j <= max_iter) {
        for (long q = 0; q < n; ++q) v[0][q] = r[q] * (1.0 / beta);
        for (int k = 0; k <= m; ++k) s[k] = 0.;
        s[0] = beta;
        for (i = 0; i < m && j <= max_iter; i++, j++) {
            A(ctx, v[i], w);
            nmv++;
            for (int k = 0; k <= i; ++k) {
                const double hk = dot(n, w, v[k]);
                H[k * ld + i] = hk;
                for (long q = 0; q < n; ++q) w[q] -= hk * v[k][q];
            }
            const double hn = sqrt(dot(n, w, w));
            H[(i + 1) * ld + i] = hn;
            for (long q = 0; q < n; ++q) v[i + 1][q] = w[q] * (1.0 / hn);
            for (int k = 0; k < i; ++k) apply_rot(&H[k * ld + i], &H[(k + 1) * ld + i], cs[k], sn[k]);
            gen_rot(H[i * ld + i], H[(i + 1) * ld + i], &cs[i], &sn[i]);
            apply_rot(&H[i * ld + i], &H[(i + 1) * ld + i], cs[i], sn[i]);
            apply_rot(&s[i], &s[i + 1], cs[i], sn[i]);
            if ((resid = fabs(s[i + 1]) / normb) < tol) {
                gm_update(n, x, i, H, ld, s, v);
                rc = 0;
                j++;
                goto done;
            }
        }
        gm_update(n, x, i - 1, H, ld, s, v);
        A(ctx, x, w);
        nmv++;
        for (long q = 0; q < n; ++q) r[q] = b[q] - w[q];
        beta = sqrt(dot(n, r, r));
        if ((resid = beta / normb) < tol) {
            rc = 0;
            goto done;
        }
    }
done:
    if (iters) *iters = j - 1;
    if (matvecs) *matvecs = nmv;
    for (int k = 0; k <= m; ++k) free(v[k]);
    free(v);
    free(H);
    free(r);
    free(w);
    return rc;
}

int orc_solve(const double *surf7, long N, double h, const double *centers, const double *charges, int M,
              const orc_bie_params *bp, double *x, double *atom_pot, double *energy, int *iters, int *matvecs) {
    bie_t B;
    bie_init(&B, surf7, N, h, bp);
    double *b = (double *)malloc(sizeof(double) * 2 * N);
    orc_rhs(surf7, N, centers, charges, M, bp, b);
    memset(x, 0, sizeof(double) * 2 * N);
    const int rc = orc_gmres(bie_apply, &B, 2 * N, x, b, bp->restart, bp->maxiter, bp->tol, iters, matvecs);
    /* polarizeMap (electric.cpp:442-485): sources = tube, targets = atoms. */
    double *dens = (double *)malloc(sizeof(double) * 4 * N);
    bie_densities(&B, x, dens);
    if (bp->mode == 0) {
        orc_tree *t = orc_tree_build(B.pts, (int)N, centers, M, bp->maxpoint, bp->maxlevel);
        double *o = (double *)malloc(sizeof(double) * 4 * M);
        orc_fmm(t, bp->np, &B.kp, ORC_KERNEL_FUSED, dens, o);
        for (int a = 0; a < M; ++a) atom_pot[a] = -o[a];
        free(o);
        orc_tree_free(t);
    } else {
        double *o = (double *)malloc(sizeof(double) * 4 * M);
        for (int k = 0; k < 4; ++k) {
            orc_tree *t = orc_tree_build(B.pts, (int)N, centers, M, bp->maxpoint, bp->maxlevel);
            orc_fmm(t, bp->np, &B.kp, k, dens + (size_t)KDENS[k] * N, o + (size_t)k * M);
            orc_tree_free(t);
        }
        for (int a = 0; a < M; ++a) atom_pot[a] = o[3 * M + a] - (o[a] + o[M + a] + o[2 * M + a]);
        free(o);
    }
    double E = 0.;
    for (int a = 0; a < M; ++a) E += atom_pot[a] * charges[a];
    *energy = 0.5 * E;
    free(dens);
    free(b);
    bie_free(&B);
    return rc;
}
