// Traveltime, amplitude and angle tables of Kirchhoff(mode='analytic' |
// 'eikonal') built on the device (pylops/waveeqprocessing/kirchhoff.py:
// 303-393 and 503-657), written straight into the operator's layouts
// (fixed-point traveltime rows, folded weight rows) with no host round trip.
//
// Every table is a row per source or receiver point, [n][ni] float64, with
// the image index ii = ix*nz + iz (2-D) or (iy*nx + ix)*nz + iz (3-D):
//  * analytic: dist^2 = (X - px)^2 + (Z - pz)^2 (+ (Y - py)^2), trav =
//    sqrt(dist^2)/v, dist = trav*v, in the reference's order of operations
//    (kirchhoff.py:576-607), so the rows equal numpy's bit for bit;
//  * eikonal (2-D and 3-D): the fast-marching equations of the package's host
//    solver (eikonal.cpp, the method scikit-fmm implements) solved by
//    Gauss-Seidel sweeps in the 4 (2-D) or 8 (3-D) diagonal orders until no
//    value changes: one CTA per table, anti-diagonal lines (planes) of the
//    sweep in parallel (their points do not neighbour one another), the same upwind
//    second-order local solver; distances (unit speed) from one table of a
//    point at the grid's corner, shifted to each point;
//  * gradients: numpy.gradient with the sample spacing (central differences
//    inside, one-sided at the ends, kirchhoff.py:642-648);
//  * angles with the vertical: atan2(dT/dx, dT/dz) in 2-D;
//    sign(dTs/dx) acos(dT/dz / |grad T|) in 3-D, where the receiver angle
//    takes the sign of the source table of the same index when ns == nr
//    (kirchhoff.py:364-393) and its own otherwise;
//  * amplitudes 1/sqrt(dist + maxdist) (2-D) or 1/(dist + maxdist) (3-D),
//    maxdist = 1e-2 (max dist_s + max dist_r) (kirchhoff.py:316-330).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "kgb_internal.h"

namespace kgb {
namespace {

// ---------------------------------------------------------------------------
// analytic rows
// ---------------------------------------------------------------------------
__global__ void analytic_kernel(const double* __restrict__ yax, const double* __restrict__ xax,
                                const double* __restrict__ zax, int ndim, int nx, int nz, int64_t ni,
                                const double* __restrict__ pts, int np, double vel, double* __restrict__ trav,
                                double* __restrict__ dist) {
    const int p = blockIdx.y;
    const double py = ndim == 3 ? pts[p] : 0.0;
    const double px = pts[(ndim - 2) * np + p];
    const double pz = pts[(ndim - 1) * np + p];
    for (int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ii < ni; ii += (int64_t)gridDim.x * blockDim.x) {
        const int iz = (int)(ii % nz);
        const int64_t r = ii / nz;
        const int ix = (int)(r % nx);
        // squares rounded before the sum (no fused multiply-add), as numpy does
        const double dxp = xax[ix] - px, dzp = zax[iz] - pz;
        double d2 = __dadd_rn(__dmul_rn(dxp, dxp), __dmul_rn(dzp, dzp));
        if (ndim == 3) {
            const double dyp = yax[r / nx] - py;
            d2 = __dadd_rn(d2, __dmul_rn(dyp, dyp));
        }
        const double t = sqrt(d2) / vel;
        trav[(size_t)p * ni + ii] = t;
        if (dist) dist[(size_t)p * ni + ii] = __dmul_rn(t, vel);
    }
}

// ---------------------------------------------------------------------------
// 2-D eikonal by diagonal Gauss-Seidel sweeps
// ---------------------------------------------------------------------------
// Times are non-negative doubles or +inf, whose order is the order of their
// bit patterns as signed 64-bit integers: the comparisons run on the integer
// pipe (the float64 pipe of this GPU runs at 1/64 of the float32 rate).
__device__ __forceinline__ bool t_less(double a, double b) {
    return __double_as_longlong(a) < __double_as_longlong(b);
}
__device__ __forceinline__ bool t_finite(double a) { return __double_as_longlong(a) < 0x7ff0000000000000LL; }

// Upwind neighbours of node k along one axis (coordinate c of n, stride st):
// the smaller finite neighbour `best`, and `second`, the node beyond it on
// the same side, when that is finite and not larger (the second-order
// stencil of the host solver, eikonal.cpp).  The negative side is taken
// first; the positive side replaces it only when strictly smaller.
__device__ __forceinline__ void ek_axis(const double* T, int64_t k, int c, int n, int64_t st, double* best,
                                        double* second, bool* have2) {
    const double vm1 = c >= 1 ? T[k - st] : INFINITY;
    const double vp1 = c + 1 < n ? T[k + st] : INFINITY;
    const double vm2 = c >= 2 ? T[k - 2 * st] : INFINITY;
    const double vp2 = c + 2 < n ? T[k + 2 * st] : INFINITY;
    *best = INFINITY;
    *have2 = false;
    if (t_finite(vm1)) {
        *best = vm1;
        if (t_finite(vm2) && !t_less(vm1, vm2)) {
            *have2 = true;
            *second = vm2;
        }
    }
    if (t_finite(vp1) && t_less(vp1, *best)) {
        *best = vp1;
        *have2 = false;
        if (t_finite(vp2) && !t_less(vp1, vp2)) {
            *have2 = true;
            *second = vp2;
        }
    }
}

// Tentative time of node (i0, i1) from its finite neighbours, reproducing
// what fast marching computes for it: marching accepts nodes in increasing
// time, so a node's neighbours become known in increasing order and its
// value is the smaller of the update with the earliest axis alone and the
// update with both axes (second order on every axis whose stencil allows
// it; the two-axis root counts when it is not below either axis' value).
// With every finite neighbour taken as known, this keeps a later (larger)
// neighbour from turning a valid second-order solve into a first-order one.
// +inf when no neighbour is finite.
//
// Each axis contributes c (T - b)^2 with c = 1/h^2, b = t1, or, second
// order, c = 9/(4 h^2), b = (4 t1 - t2)/3.  The equation is solved for
// d = T - r, r the smaller axis value, in float: d and the b - r are of
// the size of one cell's traveltime, whatever the time itself, so float
// keeps T to ~5e-8 of its size (measured against the same update in
// float64 on the 800 x 300 workload: 4.9e-8 of the largest time), and the
// float64 pipe only forms the differences b - r and the final r + d.
// Single axis: the larger root of c (d - b)^2 = rhs, b + sqrt(rhs/c).
// Two axes: A d^2 - 2 B d + C = 0 with A = c0 + c1, B = c0 b0 + c1 b1,
// C = c0 b0^2 + c1 b1^2 - rhs.
__device__ double ek_update(const double* T, int n0, int n1, float ih0, float ih1, int i0, int i1, float rhs) {
    const int64_t k = (int64_t)i0 * n1 + i1;
    double bx, sx = 0.0, bz, sz = 0.0;
    bool hx, hz;
    ek_axis(T, k, i0, n0, n1, &bx, &sx, &hx);
    ek_axis(T, k, i1, n1, 1, &bz, &sz, &hz);
    const bool fx = t_finite(bx), fz = t_finite(bz);
    if (!fx && !fz) return INFINITY;
    // axis "e" (earliest: the smaller value; axis 0 on ties) and axis "l"
    const bool zfirst = fz && (!fx || t_less(bz, bx));
    const double r = zfirst ? bz : bx;
    const double se = zfirst ? sz : sx;
    const bool he = zfirst ? hz : hx;
    const float ihe = zfirst ? ih1 : ih0;
    const float ce = he ? 2.25f * ihe : ihe;
    const float be = he ? (float)(r - se) * (1.f / 3.f) : 0.f;
    float d = be + sqrtf(rhs / ce);  // earliest axis alone
    if (fx && fz) {
        const double bl = zfirst ? bx : bz, sl = zfirst ? sx : sz;
        const bool hl = zfirst ? hx : hz;
        const float ihl = zfirst ? ih0 : ih1;
        const float dl = (float)(bl - r);
        const float cl = hl ? 2.25f * ihl : ihl;
        const float b2 = hl ? (4.f * dl - (float)(sl - r)) * (1.f / 3.f) : dl;
        const float A = ce + cl;
        const float B = ce * be + cl * b2;
        const float C = ce * be * be + cl * b2 * b2 - rhs;
        const float disc = B * B - A * C;
        if (disc >= 0.f) {
            const float t = (B + sqrtf(disc)) / A;
            if (t >= fmaxf(be, b2) && t < d) d = t;
        }
    }
    return r + (double)d;
}

constexpr int kEikThreads = 320;
constexpr int kEikMaxSets = 64;  // sweep sets before giving up (each set is 4 sweeps)

// rhs of the eikonal equation, 1/speed^2, rounded once to float
__global__ void ek_rhs_kernel(const double* __restrict__ speed, int64_t n, float* __restrict__ rhs) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = speed[i];
        rhs[i] = (float)(1.0 / (v * v));
    }
}

// One CTA per table.  CTAs [0, ns) solve the traveltimes of the sources,
// [ns, ns + nr) those of the receivers (grid points pts[2b], pts[2b + 1]),
// and CTA ns + nr the unit-speed table of a point at the grid's corner.
__global__ void __launch_bounds__(kEikThreads, 4)
eikonal_sweep_kernel(int n0, int n1, double h0, double h1, const double* __restrict__ speed,
                     const float* __restrict__ rhs, const int* __restrict__ pts, int ns, int nr, double* trav_s,
                     double* trav_r, double* corner, unsigned* __restrict__ err) {
    const int b = blockIdx.x;
    const bool unit = b >= ns + nr;
    double* T = unit ? corner : b < ns ? trav_s + (size_t)b * n0 * n1 : trav_r + (size_t)(b - ns) * n0 * n1;
    // T is read and written by all threads between barriers
    const int s0 = unit ? 0 : pts[2 * b], s1 = unit ? 0 : pts[2 * b + 1];
    const int64_t N = (int64_t)n0 * n1;
    const double r0 = 0.5 / sqrt(1.0 / (h0 * h0) + 1.0 / (h1 * h1));
    const float ih0 = (float)(1.0 / (h0 * h0)), ih1 = (float)(1.0 / (h1 * h1));
    auto spd = [&](int64_t i) { return unit ? 1.0 : speed[i]; };
    // the point and its axis neighbours start on the level set (half a cell
    // from the point); they never change
    auto frozen = [&](int i0, int i1) { return abs(i0 - s0) + abs(i1 - s1) <= 1; };
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
        const int i0 = (int)(i / n1), i1 = (int)(i - (int64_t)i0 * n1);
        double v = INFINITY;
        if (i0 == s0 && i1 == s1) v = r0 / spd(i);
        else if (frozen(i0, i1)) v = 0.5 * (i0 != s0 ? h0 : h1) / spd(i);
        T[i] = v;
    }
    __shared__ int changed;
    int sets = 0;
    for (;;) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int dir = 0; dir < 4; ++dir) {
            const bool f0 = dir == 0 || dir == 3;  // i0 increasing
            const bool f1 = dir < 2;               // i1 increasing
            for (int d = 0; d < n0 + n1 - 1; ++d) {
                // points with u0 + u1 = d, u = the sweep's coordinates
                const int lo = max(0, d - (n0 - 1)), hi = min(d, n1 - 1);
                for (int u1 = lo + (int)threadIdx.x; u1 <= hi; u1 += blockDim.x) {
                    const int u0 = d - u1;
                    const int i0 = f0 ? u0 : n0 - 1 - u0;
                    const int i1 = f1 ? u1 : n1 - 1 - u1;
                    if (frozen(i0, i1)) continue;
                    const int64_t k = (int64_t)i0 * n1 + i1;
                    const double t = ek_update(T, n0, n1, ih0, ih1, i0, i1, unit ? 1.f : rhs[k]);
                    if (t_less(t, T[k])) {
                        T[k] = t;
                        changed = 1;
                    }
                }
                __syncthreads();
            }
        }
        const int c = changed;
        __syncthreads();
        if (!c) break;
        if (++sets >= kEikMaxSets) {
            if (threadIdx.x == 0) atomicExch(err, 3u);
            break;
        }
    }
}

// 3-D: the same emulation of fast marching with up to three axes, sorted by
// their values e1 <= e2 <= e3 (ties: lower axis first): the smallest of the
// updates with {e1}, {e1, e2} and {e1, e2, e3}, each second order where the
// stencil allows it and counting when the root is not below any axis value
// (what marching computes as those neighbours are accepted in turn).  Same
// float form relative to r = the e1 value.
__device__ double ek_update3(const double* T, const int* n, const int64_t* st, const float* ih, const int* c,
                             float rhs) {
    const int64_t k = c[0] * st[0] + c[1] * st[1] + c[2] * st[2];
    double b[3], s2[3] = {0.0, 0.0, 0.0};
    bool h2[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) ek_axis(T, k, c[a], n[a], st[a], &b[a], &s2[a], &h2[a]);
    int idx[3], m = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a)
        if (t_finite(b[a])) idx[m++] = a;
    if (m == 0) return INFINITY;
    // insertion sort of the finite axes by value (stable: ties keep axis order)
    for (int i = 1; i < m; ++i)
        for (int j = i; j > 0 && t_less(b[idx[j]], b[idx[j - 1]]); --j) {
            const int t = idx[j];
            idx[j] = idx[j - 1];
            idx[j - 1] = t;
        }
    const double r = b[idx[0]];
    float cc[3], bb[3];
    for (int i = 0; i < m; ++i) {
        const int a = idx[i];
        const float d1 = (float)(b[a] - r);
        cc[i] = h2[a] ? 2.25f * ih[a] : ih[a];
        bb[i] = h2[a] ? (4.f * d1 - (float)(s2[a] - r)) * (1.f / 3.f) : d1;
    }
    float d = bb[0] + sqrtf(rhs / cc[0]);
    for (int q = 2; q <= m; ++q) {
        float A = 0.f, B = 0.f, C = -rhs, bm = -INFINITY;
        for (int i = 0; i < q; ++i) {
            A += cc[i];
            B += cc[i] * bb[i];
            C += cc[i] * bb[i] * bb[i];
            bm = fmaxf(bm, bb[i]);
        }
        const float disc = B * B - A * C;
        if (disc >= 0.f) {
            const float t = (B + sqrtf(disc)) / A;
            if (t >= bm && t < d) d = t;
        }
    }
    return r + (double)d;
}

constexpr int kEik3Threads = 512;

// 3-D tables: CTAs as in the 2-D kernel (sources, receivers, unit-speed
// corner); anti-diagonal planes u0 + u1 + u2 = d of the 8 sweep orders.
__global__ void __launch_bounds__(kEik3Threads, 2)
eikonal3_sweep_kernel(int n0, int n1, int n2, double h0, double h1, double h2, const double* __restrict__ speed,
                      const float* __restrict__ rhs, const int* __restrict__ pts, int ns, int nr, double* trav_s,
                      double* trav_r, double* corner, unsigned* __restrict__ err) {
    const int bidx = blockIdx.x;
    const bool unit = bidx >= ns + nr;
    const int64_t N = (int64_t)n0 * n1 * n2;
    double* T = unit ? corner : bidx < ns ? trav_s + (size_t)bidx * N : trav_r + (size_t)(bidx - ns) * N;
    const int p0 = unit ? 0 : pts[3 * bidx], p1 = unit ? 0 : pts[3 * bidx + 1], p2 = unit ? 0 : pts[3 * bidx + 2];
    const int n[3] = {n0, n1, n2};
    const int64_t st[3] = {(int64_t)n1 * n2, n2, 1};
    const double hh[3] = {h0, h1, h2};
    const float ih[3] = {(float)(1.0 / (h0 * h0)), (float)(1.0 / (h1 * h1)), (float)(1.0 / (h2 * h2))};
    const double r0 = 0.5 / sqrt(1.0 / (h0 * h0) + 1.0 / (h1 * h1) + 1.0 / (h2 * h2));
    auto spd = [&](int64_t i) { return unit ? 1.0 : speed[i]; };
    auto dist1 = [&](int c0, int c1, int c2) { return abs(c0 - p0) + abs(c1 - p1) + abs(c2 - p2); };
    for (int64_t i = threadIdx.x; i < N; i += blockDim.x) {
        const int c0 = (int)(i / st[0]);
        const int64_t rem = i - (int64_t)c0 * st[0];
        const int c1 = (int)(rem / n2), c2 = (int)(rem - (int64_t)c1 * n2);
        const int dd = dist1(c0, c1, c2);
        double v = INFINITY;
        if (dd == 0) v = r0 / spd(i);
        else if (dd == 1) v = 0.5 * (c0 != p0 ? hh[0] : c1 != p1 ? hh[1] : hh[2]) / spd(i);
        T[i] = v;
    }
    __shared__ int changed;
    int sets = 0;
    for (;;) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int dir = 0; dir < 8; ++dir) {
            const bool f0 = dir & 1, f1 = (dir >> 1) & 1, f2 = (dir >> 2) & 1;
            for (int d = 0; d <= n0 + n1 + n2 - 3; ++d) {
                // points of the plane: u1 in [lo1, hi1], u2 over [0, n2), u0 = d - u1 - u2 in range
                const int lo1 = max(0, d - (n0 - 1) - (n2 - 1)), hi1 = min(d, n1 - 1);
                const int64_t cnt = (int64_t)(hi1 - lo1 + 1) * n2;
                for (int64_t j = threadIdx.x; j < cnt; j += blockDim.x) {
                    const int u1 = lo1 + (int)(j / n2), u2 = (int)(j - (int64_t)(u1 - lo1) * n2);
                    const int u0 = d - u1 - u2;
                    if (u0 < 0 || u0 >= n0) continue;
                    int c[3] = {f0 ? u0 : n0 - 1 - u0, f1 ? u1 : n1 - 1 - u1, f2 ? u2 : n2 - 1 - u2};
                    if (dist1(c[0], c[1], c[2]) <= 1) continue;
                    const int64_t k = c[0] * st[0] + c[1] * st[1] + c[2];
                    const double t = ek_update3(T, n, st, ih, c, unit ? 1.f : rhs[k]);
                    if (t_less(t, T[k])) {
                        T[k] = t;
                        changed = 1;
                    }
                }
                __syncthreads();
            }
        }
        const int cflag = changed;
        __syncthreads();
        if (!cflag) break;
        if (++sets >= kEikMaxSets) {
            if (threadIdx.x == 0) atomicExch(err, 3u);
            break;
        }
    }
}

// 3-D distance rows from the corner table: row p at (i0, i1, i2) is the
// corner table at (|i0 - p0|, |i1 - p1|, |i2 - p2|).
__global__ void distance3_rows_kernel(int n0, int n1, int n2, const double* __restrict__ corner,
                                      const int* __restrict__ pts, int ns, double* __restrict__ dist_s,
                                      double* __restrict__ dist_r) {
    const int p = blockIdx.y;
    const int q0 = pts[3 * p], q1 = pts[3 * p + 1], q2 = pts[3 * p + 2];
    const int64_t N = (int64_t)n0 * n1 * n2, s0 = (int64_t)n1 * n2;
    double* out = p < ns ? dist_s + (size_t)p * N : dist_r + (size_t)(p - ns) * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int i0 = (int)(i / s0);
        const int64_t rem = i - (int64_t)i0 * s0;
        const int i1 = (int)(rem / n2), i2 = (int)(rem - (int64_t)i1 * n2);
        out[i] = corner[(int64_t)abs(i0 - q0) * s0 + (int64_t)abs(i1 - q1) * n2 + abs(i2 - q2)];
    }
}

// Unit-speed (distance) rows: with unit speed the sweeps' solution depends
// only on the offset from the point (every update reads the upwind side,
// which lies between the node and the point, inside the grid), so row p at
// (i0, i1) is the corner table at (|i0 - p0|, |i1 - p1|).  The same holds
// for the host fast-marching solver; both were checked bit for bit against
// per-point solves on the 800 x 300 grid.
__global__ void distance_rows_kernel(int n0, int n1, const double* __restrict__ corner, const int* __restrict__ pts,
                                     int ns, double* __restrict__ dist_s, double* __restrict__ dist_r) {
    const int p = blockIdx.y;
    const int p0 = pts[2 * p], p1 = pts[2 * p + 1];
    const int64_t N = (int64_t)n0 * n1;
    double* out = p < ns ? dist_s + (size_t)p * N : dist_r + (size_t)(p - ns) * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int i0 = (int)(i / n1), i1 = (int)(i - (int64_t)i0 * n1);
        out[i] = corner[(int64_t)abs(i0 - p0) * n1 + abs(i1 - p1)];
    }
}

// ---------------------------------------------------------------------------
// gradients, angles, amplitudes, folded weights
// ---------------------------------------------------------------------------
// numpy.gradient of row f along axis a (stride st, length n, spacing h) at
// coordinate c: central difference inside, one-sided at the ends
__device__ __forceinline__ double grad1(const double* __restrict__ f, int64_t k, int c, int n, int64_t st, double h) {
    if (n < 2) return 0.0;
    if (c == 0) return (f[k + st] - f[k]) / h;
    if (c == n - 1) return (f[k] - f[k - st]) / h;
    return (f[k + st] - f[k - st]) / (2.0 * h);
}

struct Geo {
    int ndim, ny, nx, nz;
    int64_t ni;
    double hy, hx, hz;
};

// gradient components of row p at ii: {d/dy, d/dx, d/dz} (3-D) or {d/dx, d/dz}
__device__ __forceinline__ void row_grad(const Geo& g, const double* __restrict__ row, int64_t ii, double* gy,
                                         double* gx, double* gz) {
    const int iz = (int)(ii % g.nz);
    const int64_t r = ii / g.nz;
    const int ix = (int)(r % g.nx);
    *gz = grad1(row, ii, iz, g.nz, 1, g.hz);
    *gx = grad1(row, ii, ix, g.nx, g.nz, g.hx);
    *gy = g.ndim == 3 ? grad1(row, ii, (int)(r / g.nx), g.ny, (int64_t)g.nx * g.nz, g.hy) : 0.0;
}

// angle of row p at every image point; sign_rows: the rows whose x-gradient
// signs the 3-D angle (the source rows for receivers when ns == nr)
__global__ void angle_kernel(Geo g, const double* __restrict__ trav, const double* __restrict__ sign_rows,
                             double* __restrict__ ang) {
    const int p = blockIdx.y;
    const double* row = trav + (size_t)p * g.ni;
    const double* srow = sign_rows + (size_t)p * g.ni;
    for (int64_t ii = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; ii < g.ni;
         ii += (int64_t)gridDim.x * blockDim.x) {
        double gy, gx, gz;
        row_grad(g, row, ii, &gy, &gx, &gz);
        double a;
        if (g.ndim == 2) {
            a = atan2(gx, gz);
        } else {
            double sy, sx, sz;
            row_grad(g, srow, ii, &sy, &sx, &sz);
            const double sg = sx > 0.0 ? 1.0 : (sx < 0.0 ? -1.0 : 0.0);
            const double nrm = __dadd_rn(__dadd_rn(__dmul_rn(gy, gy), __dmul_rn(gx, gx)), __dmul_rn(gz, gz));
            a = sg * acos(gz / sqrt(nrm));
        }
        ang[(size_t)p * g.ni + ii] = a;
    }
}

// numpy/CPython float floor division (as the angle taper index uses it)
__device__ double py_floordiv_d(double a, double b) {
    const double mod = fmod(a, b);
    double div = (a - mod) / b;
    if (mod != 0.0 && ((b < 0) != (mod < 0))) div -= 1.0;
    double fl;
    if (div != 0.0) {
        fl = floor(div);
        if (div - fl > 0.5) fl += 1.0;
    } else {
        fl = copysign(0.0, a / b);
    }
    return fl;
}

struct FoldArgs {
    double maxdist, amin, amax;
    const double* taper;  // 21 values
    int ndim;
};

// amplitude and angle taper folded with the half-angle cosines/sines into
// the operator's float32 weight rows (as the host upload does)
__global__ void fold_kernel(FoldArgs f, const double* __restrict__ dist, const double* __restrict__ ang,
                            int64_t n, float* __restrict__ wc, float* __restrict__ ws,
                            unsigned long long* __restrict__ wabs) {
    double mx = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double a = ang[k];
        const double dd = dist[k] + f.maxdist;
        const double A = f.ndim == 2 ? 1.0 / sqrt(dd) : 1.0 / dd;
        const double aa = fabs(a);
        double tap = 0.0;
        if (aa < f.amax) {
            tap = 1.0;
            if (aa >= f.amin) {
                long idx = (long)py_floordiv_d(20.0 * (aa - f.amin), f.amax - f.amin);
                idx = idx < 0 ? 0 : (idx > 20 ? 20 : idx);
                tap = f.taper[idx];
            }
        }
        const double base = A * tap;
        const float c = (float)(base * cos(a / 2.0)), s = (float)(base * sin(a / 2.0));
        wc[k] = c;
        ws[k] = s;
        mx = fmax(mx, sqrt(__dadd_rn(__dmul_rn((double)c, (double)c), __dmul_rn((double)s, (double)s))));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0 && mx > 0.0) atomicMax(wabs, (unsigned long long)__double_as_longlong(mx));
}

// ---------------------------------------------------------------------------
// reductions and quantisation
// ---------------------------------------------------------------------------
// max of |x| over n values into bits of a non-negative double (*out, zeroed)
__global__ void absmax_kernel(const double* __restrict__ x, int64_t n, unsigned long long* __restrict__ out) {
    double m = 0.0;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(x[k]));
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// non-finite values: the flat index of one in *bad (atomicMax; -1 if none)
__global__ void finite_kernel(const double* __restrict__ x, int64_t n, long long* __restrict__ bad) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(x[k])) atomicMax(bad, (long long)k);
}

// fixed-point rows: q = rint(t * inv_dt * 2^F), and the smallest q (*qmin)
__global__ void quantise_kernel(const double* __restrict__ t, int64_t n, double inv_dt, double scale,
                                int32_t* __restrict__ q, int* __restrict__ qmin) {
    int mn = INT32_MAX;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const int32_t v = (int32_t)__double2ll_rn(t[k] * inv_dt * scale);
        q[k] = v;
        mn = min(mn, v);
    }
    for (int o = 16; o > 0; o >>= 1) mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    if ((threadIdx.x & 31) == 0) atomicMin(qmin, mn);
}

// amplitude rows from distance rows: 1/sqrt(d + maxdist) (2-D), 1/(d + maxdist) (3-D)
__global__ void amplitude_kernel(const double* __restrict__ dist, int64_t n, double maxdist, int ndim,
                                 double* __restrict__ amp) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double dd = dist[k] + maxdist;
        amp[k] = ndim == 2 ? 1.0 / sqrt(dd) : 1.0 / dd;
    }
}

__global__ void vscale_kernel(const double* __restrict__ vel, int64_t nvel, int64_t ni, float* __restrict__ vs) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < ni; k += (int64_t)gridDim.x * blockDim.x)
        vs[k] = (float)(2.0 / vel[nvel == 1 ? 0 : k]);
}

// [n][ni] rows -> (ni, n) reference layout
__global__ void transpose_kernel(const double* __restrict__ rows, int n, int64_t ni, double* __restrict__ out) {
    __shared__ double tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32;
    const int j0 = blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int j = j0 + r;
        const int64_t i = i0 + threadIdx.x;
        if (j < n && i < ni) tile[r][threadIdx.x] = rows[(size_t)j * ni + i];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + r;
        const int j = j0 + threadIdx.x;
        if (j < n && i < ni) out[(size_t)i * n + j] = tile[threadIdx.x][r];
    }
}

}  // namespace
}  // namespace kgb

// ---------------------------------------------------------------------------
// launchers (declared in kgb_internal.h)
// ---------------------------------------------------------------------------
namespace kgb {

static int grid_for(int64_t n) {
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (int)std::min<int64_t>((n + 255) / 256, (int64_t)std::max(sms, 1) * 8);
}

int launch_analytic_rows(const TableGeom& g, const double* yax, const double* xax, const double* zax,
                         const double* pts, int np, double vel, double* trav, double* dist, cudaStream_t s) {
    dim3 grid((unsigned)std::max(1, grid_for(g.ni) / std::max(1, np / 8 + 1)), (unsigned)np);
    analytic_kernel<<<grid, 256, 0, s>>>(yax, xax, zax, g.ndim, g.nx, g.nz, g.ni, pts, np, vel, trav, dist);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_eikonal_tables(const TableGeom& g, const double* speed, float* rhs, const int* pts, int ns, int nr,
                          double* trav_s, double* trav_r, double* corner, unsigned* err, cudaStream_t s) {
    ek_rhs_kernel<<<grid_for(g.ni), 256, 0, s>>>(speed, g.ni, rhs);
    KGB_CUDA_TRY(cudaGetLastError());
    if (g.ndim == 2) {
        eikonal_sweep_kernel<<<ns + nr + 1, kEikThreads, 0, s>>>(g.nx, g.nz, g.hx, g.hz, speed, rhs, pts, ns, nr,
                                                                  trav_s, trav_r, corner, err);
    } else {
        eikonal3_sweep_kernel<<<ns + nr + 1, kEik3Threads, 0, s>>>(g.ny, g.nx, g.nz, g.hy, g.hx, g.hz, speed, rhs, pts,
                                                                    ns, nr, trav_s, trav_r, corner, err);
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_distance_rows(const TableGeom& g, const double* corner, const int* pts, int ns, int nr, double* dist_s,
                         double* dist_r, cudaStream_t s) {
    dim3 grid((unsigned)std::max(1, grid_for(g.ni) / std::max(1, (ns + nr) / 8 + 1)), (unsigned)(ns + nr));
    if (g.ndim == 2) distance_rows_kernel<<<grid, 256, 0, s>>>(g.nx, g.nz, corner, pts, ns, dist_s, dist_r);
    else distance3_rows_kernel<<<grid, 256, 0, s>>>(g.ny, g.nx, g.nz, corner, pts, ns, dist_s, dist_r);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_angle_rows(const TableGeom& g, const double* trav, const double* sign_rows, int np, double* ang,
                      cudaStream_t s) {
    Geo geo{g.ndim, g.ny, g.nx, g.nz, g.ni, g.hy, g.hx, g.hz};
    dim3 grid((unsigned)std::max(1, grid_for(g.ni) / std::max(1, np / 8 + 1)), (unsigned)np);
    angle_kernel<<<grid, 256, 0, s>>>(geo, trav, sign_rows ? sign_rows : trav, ang);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_fold_rows(int ndim, double maxdist, double amin, double amax, const double* taper21,
                     const double* dist, const double* ang, int64_t n, float* wc, float* ws,
                     unsigned long long* wabs, cudaStream_t s) {
    FoldArgs f{maxdist, amin, amax, taper21, ndim};
    fold_kernel<<<grid_for(n), 256, 0, s>>>(f, dist, ang, n, wc, ws, wabs);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_absmax(const double* x, int64_t n, unsigned long long* out, cudaStream_t s) {
    absmax_kernel<<<grid_for(n), 256, 0, s>>>(x, n, out);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_finite_check(const double* x, int64_t n, long long* bad, cudaStream_t s) {
    finite_kernel<<<grid_for(n), 256, 0, s>>>(x, n, bad);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_quantise(const double* t, int64_t n, double inv_dt, double scale, int32_t* q, int* qmin, cudaStream_t s) {
    quantise_kernel<<<grid_for(n), 256, 0, s>>>(t, n, inv_dt, scale, q, qmin);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_vscale(const double* vel, int64_t nvel, int64_t ni, float* vs, cudaStream_t s) {
    vscale_kernel<<<grid_for(ni), 256, 0, s>>>(vel, nvel, ni, vs);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_amplitude_rows(const double* dist, int64_t n, double maxdist, int ndim, double* amp, cudaStream_t s) {
    amplitude_kernel<<<grid_for(n), 256, 0, s>>>(dist, n, maxdist, ndim, amp);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int launch_rows_to_reference(const double* rows, int n, int64_t ni, double* out, cudaStream_t s) {
    dim3 grid((unsigned)((ni + 31) / 32), (unsigned)((n + 31) / 32));
    transpose_kernel<<<grid, dim3(32, 8), 0, s>>>(rows, n, ni, out);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

}  // namespace kgb
