/*
 * C restatement of the reference's Numba CPU engine for the Kirchhoff path.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the CUDA kernels at sizes the
 * NumPy oracle cannot reach, and the timed CPU baseline of bench.py.  The
 * product never links or calls this file.
 *
 * It follows the loop nests of pylops/waveeqprocessing/kirchhoff.py, which
 * the reference JIT-compiles with numba (nopython, nogil, parallel) at
 * kirchhoff.py:1003-1018:
 *   forward  _travsrcrec_kirch_matvec   kirchhoff.py:728-752  prange over isrc
 *            _ampsrcrec_kirch_matvec    kirchhoff.py:784-889  prange over isrc
 *   adjoint  _travsrcrec_kirch_rmatvec  kirchhoff.py:755-781  prange over ii
 *            _ampsrcrec_kirch_rmatvec   kirchhoff.py:892-1001 prange over ii
 * in float64, tables in the reference layout (ni, ns) / (ni, nr), plus the
 * 'same' wavelet convolution of convolve1d.py:57-116 restated as a direct
 * FIR.  OpenMP threads play the role of numba's prange.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int ns, nr, nt, nz;
    int64_t ni;
    double dt;
    const double *ts, *tr;         /* (ni, ns), (ni, nr) */
    int dynamic;
    const double *as, *ar;         /* amplitudes */
    const double *ans, *anr;       /* angles */
    const double *vel;             /* (ni) */
    double apmin, apmax, amin, amax;
    const double *taper;           /* 21 */
    const int64_t *six, *rix;      /* (ns*nr) */
} ko_op;

/* numpy/CPython float floor division */
static double floordiv(double a, double b) {
    double mod = fmod(a, b), div, fl;
    if (b == 0.0) return a / b;
    div = (a - mod) / b;
    if (mod != 0.0 && ((b < 0) != (mod < 0))) div -= 1.0;
    if (div != 0.0) {
        fl = floor(div);
        if (div - fl > 0.5) fl += 1.0;
    } else {
        fl = copysign(0.0, a / b);
    }
    return fl;
}

/* damp * aptap of kirchhoff.py:820-880 in *out; returns 0 when the angle or
 * offset aperture rejects the pair-point */
static int dyn_weight(const ko_op* K, int64_t ii, int is, int ir, double* out) {
    const double a_s = K->ans[ii * K->ns + is], a_r = K->anr[ii * K->nr + ir];
    const double damp = 2.0 * cos((a_s - a_r) / 2.0) * K->as[ii * K->ns + is] * K->ar[ii * K->nr + ir] / K->vel[ii];
    const double dang = K->amax - K->amin, dap = K->apmax - K->apmin;
    const double abs_s = fabs(a_s), abs_r = fabs(a_r);
    double aptap = 1.0, ap;
    int64_t pair = (int64_t)is * K->nr + ir;
    int iz = (int)(ii % K->nz);
    if (!(abs_s < K->amax && abs_r < K->amax)) return 0;
    if (abs_s >= K->amin) aptap *= K->taper[(int)floordiv(20 * (abs_s - K->amin), dang)];
    if (abs_r >= K->amin) aptap *= K->taper[(int)floordiv(20 * (abs_r - K->amin), dang)];
    ap = fabs((double)(K->six[pair] - K->rix[pair])) / (iz + 1);
    if (!(ap < K->apmax)) return 0;
    if (ap >= K->apmin) aptap *= K->taper[(int)(20 * floordiv(ap - K->apmin, dap))];
    *out = damp * aptap;
    return 1;
}

/* Forward spreading into y (ns*nr, nt), zeroed by the caller; sources
 * [s0, s1) only (a bounded sample of the full operator). */
void ko_spread(const ko_op* K, const double* x, double* y, int s0, int s1) {
    const int nt = K->nt;
    int is;
#pragma omp parallel for schedule(dynamic, 1)
    for (is = s0; is < s1; ++is) {
        for (int ir = 0; ir < K->nr; ++ir) {
            double* row = y + ((int64_t)is * K->nr + ir) * nt;
            for (int64_t ii = 0; ii < K->ni; ++ii) {
                const double t = K->ts[ii * K->ns + is] + K->tr[ii * K->nr + ir];
                const double tt = t / K->dt;
                const int it = (int)tt;
                const double w = tt - it;
                double v = x[ii];
                if (K->dynamic) {
                    double wt;
                    if (!dyn_weight(K, ii, is, ir, &wt)) continue;
                    v *= wt;
                }
                if (0 <= it && it < nt - 1) {
                    row[it] += v * (1 - w);
                    row[it + 1] += v * w;
                }
            }
        }
    }
}

/* Adjoint gathering from d (ns*nr, nt) into img (ni); sources [s0, s1). */
void ko_gather(const ko_op* K, const double* d, double* img, int s0, int s1) {
    const int nt = K->nt;
    int64_t ii;
#pragma omp parallel for schedule(static)
    for (ii = 0; ii < K->ni; ++ii) {
        double acc = 0.0;
        for (int is = s0; is < s1; ++is) {
            for (int ir = 0; ir < K->nr; ++ir) {
                const double t = K->ts[ii * K->ns + is] + K->tr[ii * K->nr + ir];
                const double tt = t / K->dt;
                const int it = (int)tt;
                const double w = tt - it;
                if (0 <= it && it < nt - 1) {
                    const double* row = d + ((int64_t)is * K->nr + ir) * nt;
                    double v = row[it] * (1 - w) + row[it + 1] * w;
                    if (K->dynamic) {
                        double wt;
                        if (!dyn_weight(K, ii, is, ir, &wt)) continue;
                        v *= wt;
                    }
                    acc += v;
                }
            }
        }
        img[ii] += acc;
    }
}

/* y[n] = sum_k h[k] x[n + (L-1)/2 - k] per trace ('same' mode). */
void ko_conv(const double* x, double* y, int64_t ntr, int nt, const double* h, int L) {
    const int c = (L - 1) / 2;
    int64_t tr;
#pragma omp parallel for schedule(static)
    for (tr = 0; tr < ntr; ++tr) {
        const double* xr = x + tr * nt;
        double* yr = y + tr * nt;
        for (int n = 0; n < nt; ++n) {
            double acc = 0.0;
            int kmin = n + c - (nt - 1);
            int kmax = n + c;
            if (kmin < 0) kmin = 0;
            if (kmax > L - 1) kmax = L - 1;
            for (int k = kmin; k <= kmax; ++k) acc += h[k] * xr[n + c - k];
            yr[n] = acc;
        }
    }
}
