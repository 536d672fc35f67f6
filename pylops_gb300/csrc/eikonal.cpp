// Fast-marching eikonal solver for the traveltime and distance tables of
// Kirchhoff(mode='eikonal') (pylops/waveeqprocessing/kirchhoff.py:609-638).
//
// The reference calls scikit-fmm once per source and receiver:
//   phi = 1 everywhere, phi[src] = -1
//   dist = skfmm.distance(phi, dx);  trav = skfmm.travel_time(phi, speed, dx)
// This file restates that published method (Sethian's fast marching with
// second-order upwind differences where the upwind stencil allows it) in
// C++ with one OpenMP thread per point source:
//  * the zero level set of phi lies half a cell from the source node along
//    each axis, so the source node starts at distance 0.5/sqrt(sum 1/h_a^2)
//    and each axis neighbour at 0.5*h_a (linear interpolation of phi);
//  * those nodes are frozen, the rest is marched in increasing arrival time
//    with |grad T| = 1/speed (speed = 1 for the distance table).
// Values are reported positive on both sides of the level set.
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <queue>
#include <vector>

#include "kgb_internal.h"

namespace {

struct Grid {
    int nd;
    int n[3];
    int64_t stride[3];
    double h[3];
    int64_t N;
};

enum : uint8_t { FAR = 0, TRIAL = 1, KNOWN = 2 };

// Solve sum_a alpha_a^2 (T - beta_a)^2 = rhs for the larger root; returns
// false when no causal root exists.
static bool solve_quadratic(int m, const double* alpha2, const double* beta, double rhs, double* T) {
    double A = 0.0, B = 0.0, C = -rhs;
    double bmax = -INFINITY;
    for (int i = 0; i < m; ++i) {
        A += alpha2[i];
        B += -2.0 * alpha2[i] * beta[i];
        C += alpha2[i] * beta[i] * beta[i];
        bmax = std::max(bmax, beta[i]);
    }
    const double disc = B * B - 4.0 * A * C;
    if (disc < 0.0) return false;
    const double t = (-B + sqrt(disc)) / (2.0 * A);
    if (t < bmax) return false;
    *T = t;
    return true;
}

static double update(const Grid& g, const double* val, const uint8_t* st, int64_t idx, const int* coord,
                     double inv_speed2, int order) {
    // per axis: the smaller known upwind neighbour (first order) and, when the
    // node behind it is known and not later, the second-order stencil
    // (3T - 4T1 + T2) / 2h
    double a2o[3], b2o[3], a1[3], b1[3];
    int m = 0;
    for (int a = 0; a < g.nd; ++a) {
        double best = INFINITY, second = INFINITY;
        bool have2 = false;
        for (int dir = -1; dir <= 1; dir += 2) {
            const int c1 = coord[a] + dir;
            if (c1 < 0 || c1 >= g.n[a]) continue;
            const int64_t i1 = idx + dir * g.stride[a];
            if (st[i1] != KNOWN) continue;
            const double v1 = val[i1];
            if (v1 < best) {
                best = v1;
                have2 = false;
                const int c2 = coord[a] + 2 * dir;
                if (order >= 2 && c2 >= 0 && c2 < g.n[a]) {
                    const int64_t i2 = idx + 2 * dir * g.stride[a];
                    if (st[i2] == KNOWN && val[i2] <= v1) {
                        have2 = true;
                        second = val[i2];
                    }
                }
            }
        }
        if (best < INFINITY) {
            const double h = g.h[a];
            a1[m] = 1.0 / (h * h);
            b1[m] = best;
            if (have2) {
                a2o[m] = 9.0 / (4.0 * h * h);
                b2o[m] = (4.0 * best - second) / 3.0;
            } else {
                a2o[m] = a1[m];
                b2o[m] = best;
            }
            ++m;
        }
    }
    double T;
    if (order >= 2 && solve_quadratic(m, a2o, b2o, inv_speed2, &T)) return T;
    // first order with all axes, then drop the latest-arriving axes
    int ord[3] = {0, 1, 2};
    std::sort(ord, ord + m, [&](int x, int y) { return b1[x] < b1[y]; });
    for (int k = m; k >= 1; --k) {
        double aa[3], bb[3];
        for (int i = 0; i < k; ++i) { aa[i] = a1[ord[i]]; bb[i] = b1[ord[i]]; }
        if (solve_quadratic(k, aa, bb, inv_speed2, &T)) return T;
    }
    return b1[ord[0]] + sqrt(inv_speed2 / a1[ord[0]]);
}

static void march(const Grid& g, const double* speed, const int* src, int order, double* val, uint8_t* st) {
    std::fill(val, val + g.N, INFINITY);
    memset(st, FAR, (size_t)g.N);
    int64_t s = 0;
    for (int a = 0; a < g.nd; ++a) s += src[a] * g.stride[a];
    double inv_h2 = 0.0;
    for (int a = 0; a < g.nd; ++a) inv_h2 += 1.0 / (g.h[a] * g.h[a]);
    auto spd = [&](int64_t i) { return speed ? speed[i] : 1.0; };
    val[s] = (0.5 / sqrt(inv_h2)) / spd(s);
    st[s] = KNOWN;
    for (int a = 0; a < g.nd; ++a)
        for (int dir = -1; dir <= 1; dir += 2) {
            const int c = src[a] + dir;
            if (c < 0 || c >= g.n[a]) continue;
            const int64_t i = s + dir * g.stride[a];
            val[i] = 0.5 * g.h[a] / spd(i);
            st[i] = KNOWN;
        }
    typedef std::pair<double, int64_t> E;
    std::priority_queue<E, std::vector<E>, std::greater<E>> heap;
    auto coords = [&](int64_t i, int* c) {
        for (int a = 0; a < g.nd; ++a) {
            c[a] = (int)((i / g.stride[a]) % g.n[a]);
        }
    };
    auto relax_neighbours = [&](int64_t i) {
        int c[3];
        coords(i, c);
        for (int a = 0; a < g.nd; ++a)
            for (int dir = -1; dir <= 1; dir += 2) {
                const int cc = c[a] + dir;
                if (cc < 0 || cc >= g.n[a]) continue;
                const int64_t j = i + dir * g.stride[a];
                if (st[j] == KNOWN) continue;
                int cj[3] = {c[0], c[1], c[2]};
                cj[a] = cc;
                const double sp = spd(j);
                const double T = update(g, val, st, j, cj, 1.0 / (sp * sp), order);
                if (T < val[j]) {
                    val[j] = T;
                    st[j] = TRIAL;
                    heap.push({T, j});
                }
            }
    };
    for (int64_t i = 0; i < g.N; ++i)
        if (st[i] == KNOWN) relax_neighbours(i);
    while (!heap.empty()) {
        const E e = heap.top();
        heap.pop();
        const int64_t i = e.second;
        if (st[i] == KNOWN || e.first != val[i]) continue;
        st[i] = KNOWN;
        relax_neighbours(i);
    }
}

}  // namespace

extern "C" int kgb_eikonal_tables(int ndim, const int* dims, const double* dsamp, const double* speed,
                                  int npts, const int* pts, double* trav_out, double* dist_out,
                                  int order, int nthreads) {
    using kgb::set_error;
    if (ndim != 2 && ndim != 3) return set_error(KGB_ERR_VALUE, "eikonal: ndim must be 2 or 3");
    if (!dims || !dsamp || !pts || !trav_out || npts <= 0)
        return set_error(KGB_ERR_VALUE, "eikonal: null argument");
    Grid g;
    g.nd = ndim;
    g.N = 1;
    for (int a = 0; a < ndim; ++a) {
        if (dims[a] < 2) return set_error(KGB_ERR_VALUE, "eikonal: each axis needs at least 2 samples");
        if (!(dsamp[a] > 0.0)) return set_error(KGB_ERR_VALUE, "eikonal: spacing must be positive");
        g.n[a] = dims[a];
        g.h[a] = dsamp[a];
        g.N *= dims[a];
    }
    g.stride[ndim - 1] = 1;
    for (int a = ndim - 2; a >= 0; --a) g.stride[a] = g.stride[a + 1] * g.n[a + 1];
    if (speed) {
        for (int64_t i = 0; i < g.N; ++i)
            if (!(speed[i] > 0.0) || !isfinite(speed[i]))
                return set_error(KGB_ERR_VALUE, "eikonal: velocity must be positive and finite");
    }
    for (int k = 0; k < npts; ++k)
        for (int a = 0; a < ndim; ++a)
            if (pts[k * ndim + a] < 0 || pts[k * ndim + a] >= g.n[a])
                return set_error(KGB_ERR_VALUE, "eikonal: point %d lies outside the grid", k);
    const int nthr = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nthr)
    {
        std::vector<double> val(g.N);
        std::vector<uint8_t> st(g.N);
#pragma omp for schedule(dynamic, 1)
        for (int k = 0; k < npts; ++k) {
            const int* src = pts + (size_t)k * ndim;
            march(g, speed, src, order, val.data(), st.data());
            for (int64_t i = 0; i < g.N; ++i) trav_out[(size_t)i * npts + k] = val[i];
            if (dist_out) {
                march(g, nullptr, src, order, val.data(), st.data());
                for (int64_t i = 0; i < g.N; ++i) dist_out[(size_t)i * npts + k] = val[i];
            }
        }
    }
    return KGB_OK;
}
