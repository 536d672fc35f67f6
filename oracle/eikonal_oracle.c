/*
 * Fast-marching traveltime and distance tables for Kirchhoff(mode='eikonal').
 *
 * TEST INFRASTRUCTURE ONLY: the oracle's eikonal tables (the reference arm of
 * bench.py builds its tables with it, and a CPU test holds the package's own
 * solver to it).  The product never links or calls this file.
 *
 * The reference (pylops/waveeqprocessing/kirchhoff.py:609-638) calls
 * scikit-fmm once per source and receiver with phi = 1 everywhere and
 * phi = -1 at the point:
 *     dist  = skfmm.distance(phi, dx)
 *     trav  = skfmm.travel_time(phi, speed=vel, dx)
 * scikit-fmm (an unpinned dependency whose source is not part of the
 * reference) implements Sethian's fast marching method with second-order
 * upwind differences where the upwind stencil allows them.  This file
 * restates that published method:
 *   1. initial front: the zero level set of phi lies half a cell from the
 *      point along every axis (linear interpolation of phi between -1 and
 *      1), so the point itself is at 1 / sqrt(sum_a (2/h_a)^2) and each of
 *      its axis neighbours at h_a / 2; those nodes are accepted, with times
 *      distance / speed;
 *   2. every node next to an accepted one gets a tentative time from the
 *      upwind quadratic  sum_a c_a (T - b_a)^2 = 1 / speed^2  built from its
 *      accepted neighbours: per axis the smaller accepted neighbour t1
 *      (c = 1/h^2, b = t1) or, when the node beyond it on the same side is
 *      accepted with t2 <= t1, the second-order stencil (3T - 4 t1 + t2)/2h
 *      (c = 9/(4 h^2), b = (4 t1 - t2)/3); the larger root counts when it is
 *      not below any b_a, else the first-order equation is solved with the
 *      axes in increasing order of t1, dropping the latest axes until a
 *      causal root exists;
 *   3. the tentative node with the smallest time (ties: smallest linear
 *      index) is accepted and its neighbours are recomputed; repeat.
 * Times are reported positive on both sides of the level set.
 *
 * The narrow band is an indexed binary heap with decrease-key; tables of
 * several points run in parallel (OpenMP), one point per thread.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

enum { ST_FAR = 0, ST_BAND = 1, ST_DONE = 2 };

typedef struct {
    int nd;
    int n[3];
    int64_t st[3]; /* strides, last axis fastest */
    double h[3];
    int64_t N;
} eg_grid;

typedef struct {
    int64_t* node;  /* heap slots -> grid index */
    int64_t* slot;  /* grid index -> heap slot, -1 when not in the heap */
    int64_t size;
    const double* t;
} eg_heap;

static int eg_before(const eg_heap* H, int64_t a, int64_t b) {
    const double ta = H->t[a], tb = H->t[b];
    return ta < tb || (ta == tb && a < b);
}

static void eg_swap(eg_heap* H, int64_t i, int64_t j) {
    int64_t a = H->node[i], b = H->node[j];
    H->node[i] = b;
    H->node[j] = a;
    H->slot[b] = i;
    H->slot[a] = j;
}

static void eg_up(eg_heap* H, int64_t i) {
    while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (!eg_before(H, H->node[i], H->node[p])) break;
        eg_swap(H, i, p);
        i = p;
    }
}

static void eg_down(eg_heap* H, int64_t i) {
    for (;;) {
        int64_t l = 2 * i + 1, r = l + 1, m = i;
        if (l < H->size && eg_before(H, H->node[l], H->node[m])) m = l;
        if (r < H->size && eg_before(H, H->node[r], H->node[m])) m = r;
        if (m == i) break;
        eg_swap(H, i, m);
        i = m;
    }
}

/* insert node k, or move it up after its time decreased */
static void eg_push_or_decrease(eg_heap* H, int64_t k) {
    if (H->slot[k] < 0) {
        H->node[H->size] = k;
        H->slot[k] = H->size;
        H->size++;
    }
    eg_up(H, H->slot[k]);
}

static int64_t eg_pop(eg_heap* H) {
    int64_t top = H->node[0];
    H->size--;
    if (H->size > 0) {
        H->node[0] = H->node[H->size];
        H->slot[H->node[0]] = 0;
        eg_down(H, 0);
    }
    H->slot[top] = -1;
    return top;
}

/* larger root of sum_i c[i] (T - b[i])^2 = rhs; 1 when it exists and is
 * not below any b[i] */
static int eg_root(int m, const double* c, const double* b, double rhs, double* T) {
    double A = 0, B = 0, C = -rhs, bmax = -INFINITY, disc, r;
    int i;
    for (i = 0; i < m; ++i) {
        A += c[i];
        B -= 2 * c[i] * b[i];
        C += c[i] * b[i] * b[i];
        if (b[i] > bmax) bmax = b[i];
    }
    disc = B * B - 4 * A * C;
    if (disc < 0) return 0;
    r = (-B + sqrt(disc)) / (2 * A);
    if (r < bmax) return 0;
    *T = r;
    return 1;
}

/* tentative time of node k at coordinates c from its accepted neighbours */
static double eg_tentative(const eg_grid* g, const double* t, const unsigned char* state, int64_t k,
                           const int* c, double slow2, int order) {
    double c2[3], b2[3], c1[3], b1[3];
    int m = 0, a, i, j;
    for (a = 0; a < g->nd; ++a) {
        int side = 0;
        double t1 = INFINITY;
        /* the smaller accepted neighbour; the lower side wins a tie */
        if (c[a] > 0 && state[k - g->st[a]] == ST_DONE) {
            side = -1;
            t1 = t[k - g->st[a]];
        }
        if (c[a] < g->n[a] - 1 && state[k + g->st[a]] == ST_DONE && t[k + g->st[a]] < t1) {
            side = 1;
            t1 = t[k + g->st[a]];
        }
        if (!side) continue;
        c1[m] = 1.0 / (g->h[a] * g->h[a]);
        b1[m] = t1;
        c2[m] = c1[m];
        b2[m] = t1;
        if (order >= 2) {
            int c_far = c[a] + 2 * side;
            if (c_far >= 0 && c_far < g->n[a]) {
                int64_t kf = k + 2 * side * g->st[a];
                if (state[kf] == ST_DONE && t[kf] <= t1) {
                    c2[m] = 2.25 / (g->h[a] * g->h[a]);
                    b2[m] = (4.0 * t1 - t[kf]) / 3.0;
                }
            }
        }
        ++m;
    }
    {
        double T;
        int idx[3] = {0, 1, 2};
        if (order >= 2 && eg_root(m, c2, b2, slow2, &T)) return T;
        /* first order, axes by increasing t1 (insertion sort of <= 3) */
        for (i = 1; i < m; ++i)
            for (j = i; j > 0 && b1[idx[j]] < b1[idx[j - 1]]; --j) {
                int s = idx[j];
                idx[j] = idx[j - 1];
                idx[j - 1] = s;
            }
        for (i = m; i >= 1; --i) {
            double cc[3], bb[3];
            for (j = 0; j < i; ++j) {
                cc[j] = c1[idx[j]];
                bb[j] = b1[idx[j]];
            }
            if (eg_root(i, cc, bb, slow2, &T)) return T;
        }
        return b1[idx[0]] + sqrt(slow2 / c1[idx[0]]);
    }
}

static void eg_coords(const eg_grid* g, int64_t k, int* c) {
    int a;
    for (a = 0; a < g->nd; ++a) c[a] = (int)((k / g->st[a]) % g->n[a]);
}

/* recompute the non-accepted neighbours of accepted node k */
static void eg_relax(const eg_grid* g, const double* speed, double* t, unsigned char* state, eg_heap* H,
                     int64_t k, int order) {
    int c[3], a, s;
    eg_coords(g, k, c);
    for (a = 0; a < g->nd; ++a)
        for (s = -1; s <= 1; s += 2) {
            int cn[3] = {c[0], c[1], c[2]};
            int64_t j;
            double sp, T;
            cn[a] += s;
            if (cn[a] < 0 || cn[a] >= g->n[a]) continue;
            j = k + s * g->st[a];
            if (state[j] == ST_DONE) continue;
            sp = speed ? speed[j] : 1.0;
            T = eg_tentative(g, t, state, j, cn, 1.0 / (sp * sp), order);
            if (T < t[j]) {
                t[j] = T;
                state[j] = ST_BAND;
                eg_push_or_decrease(H, j);
            }
        }
}

static void eg_march(const eg_grid* g, const double* speed, const int* p, int order, double* t,
                     unsigned char* state, eg_heap* H) {
    int64_t k0 = 0, k;
    double q = 0;
    int a, s;
    for (k = 0; k < g->N; ++k) {
        t[k] = INFINITY;
        H->slot[k] = -1;
    }
    memset(state, ST_FAR, (size_t)g->N);
    H->size = 0;
    for (a = 0; a < g->nd; ++a) {
        k0 += p[a] * g->st[a];
        q += 4.0 / (g->h[a] * g->h[a]);
    }
    t[k0] = (1.0 / sqrt(q)) / (speed ? speed[k0] : 1.0);
    state[k0] = ST_DONE;
    for (a = 0; a < g->nd; ++a)
        for (s = -1; s <= 1; s += 2) {
            int cn = p[a] + s;
            int64_t j;
            if (cn < 0 || cn >= g->n[a]) continue;
            j = k0 + s * g->st[a];
            t[j] = 0.5 * g->h[a] / (speed ? speed[j] : 1.0);
            state[j] = ST_DONE;
        }
    for (k = 0; k < g->N; ++k)
        if (state[k] == ST_DONE) eg_relax(g, speed, t, state, H, k, order);
    while (H->size > 0) {
        k = eg_pop(H);
        state[k] = ST_DONE;
        eg_relax(g, speed, t, state, H, k, order);
    }
}

/* Tables of npts points on a grid of nd (2 or 3) axes, sizes n, spacings h,
 * last axis fastest.  pts: (npts, nd) grid coordinates.  trav (may be NULL)
 * gets the traveltimes with `speed` (N values), dist (may be NULL) the
 * distances (speed 1); both laid out (N, npts) like the reference's tables.
 * Returns 0, or -1 on a bad argument or a failed allocation. */
int eo_tables(int nd, const int* n, const double* h, const double* speed, int npts, const int* pts,
              double* trav, double* dist, int order) {
    eg_grid g;
    int a, k, bad = 0;
    if (nd < 2 || nd > 3 || npts <= 0) return -1;
    g.nd = nd;
    g.N = 1;
    for (a = 0; a < nd; ++a) {
        if (n[a] < 2 || !(h[a] > 0)) return -1;
        g.n[a] = n[a];
        g.h[a] = h[a];
        g.N *= n[a];
    }
    g.st[nd - 1] = 1;
    for (a = nd - 2; a >= 0; --a) g.st[a] = g.st[a + 1] * g.n[a + 1];
    for (k = 0; k < npts; ++k)
        for (a = 0; a < nd; ++a)
            if (pts[k * nd + a] < 0 || pts[k * nd + a] >= n[a]) return -1;
#pragma omp parallel reduction(| : bad)
    {
        double* t = (double*)malloc(sizeof(double) * g.N);
        unsigned char* state = (unsigned char*)malloc((size_t)g.N);
        eg_heap H;
        H.node = (int64_t*)malloc(sizeof(int64_t) * g.N);
        H.slot = (int64_t*)malloc(sizeof(int64_t) * g.N);
        H.t = t;
        const int ok = t && state && H.node && H.slot;
        int kk;
        if (!ok) bad = 1;
#pragma omp for schedule(dynamic, 1)
        for (kk = 0; kk < npts; ++kk) {
            int64_t i;
            if (!ok) continue;
            if (trav) {
                eg_march(&g, speed, pts + (size_t)kk * nd, order, t, state, &H);
                for (i = 0; i < g.N; ++i) trav[i * npts + kk] = t[i];
            }
            if (dist) {
                eg_march(&g, NULL, pts + (size_t)kk * nd, order, t, state, &H);
                for (i = 0; i < g.N; ++i) dist[i * npts + kk] = t[i];
            }
        }
        free(t);
        free(state);
        free(H.node);
        free(H.slot);
    }
    return bad ? -1 : 0;
}
