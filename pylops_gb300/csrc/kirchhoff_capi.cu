// C ABI of the Kirchhoff operator (include/kirchhoff_gb300.h): handle
// life cycle, table upload (quantisation to fixed point, folding of the
// dynamic weights) and the apply entry points.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fixed_acc.cuh"
#include "kgb_internal.h"

namespace kgb {

static thread_local std::string g_last_error;

int set_error(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_error(cudaError_t e, const char* what) {
    return set_error(e == cudaErrorMemoryAllocation ? KGB_ERR_MEMORY : KGB_ERR_CUDA, "%s: %s (%s)",
                     what, cudaGetErrorString(e), cudaGetErrorName(e));
}

template <typename T>
static int dev_alloc(T** p, size_t n, const char* what) {
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    if (n == 0) return KGB_OK;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_error(e, what);
    }
    return KGB_OK;
}

// numpy/CPython float floor division (npy_divmod), so that taper indices are
// computed exactly as `a // b` is in the reference's loops.
static double py_floordiv(double a, double b) {
    if (b == 0.0) return a / b;
    double mod = fmod(a, b);
    double div = (a - mod) / b;
    if (mod != 0.0) {
        if ((b < 0) != (mod < 0)) div -= 1.0;
    }
    double fl;
    if (div != 0.0) {
        fl = floor(div);
        if (div - fl > 0.5) fl += 1.0;
    } else {
        fl = copysign(0.0, a / b);
    }
    return fl;
}

// Fractional bits of the fixed-point traveltime: the largest F such that
// every table entry and nt fit with headroom for the sum of two entries in
// an int32 (|q| < 2^30), capped at 22.
static int choose_frac_bits(double max_samples, int nt) {
    auto bits_for = [](double v) {
        int b = 0;
        while (b < 62 && ldexp(1.0, b) < v) ++b;
        return b;
    };
    int need = std::max(bits_for(max_samples + 2.0), bits_for((double)nt + 1.0));
    return std::min(22, 30 - need);
}

// Dynamic-mode records {tq, wc, ws} from the traveltime and weight arrays;
// run whenever either side changes.
static int repack(kgb_kirchhoff* op) {
    if (!op->dynamic || !op->trav_ready || !op->dyn_ready) return KGB_OK;
    int rc;
    if (!op->stab && (rc = dev_alloc(&op->stab, (size_t)op->ns * op->ni, "alloc source records"))) return rc;
    if (!op->rtab && (rc = dev_alloc(&op->rtab, (size_t)op->nr * op->ni, "alloc receiver records"))) return rc;
    const int64_t ncol = op->ni / op->nz;
    if (!op->srng && (rc = dev_alloc(&op->srng, (size_t)op->ns * ncol, "alloc source ranges"))) return rc;
    if (!op->rrng && (rc = dev_alloc(&op->rrng, (size_t)op->nr * ncol, "alloc receiver ranges"))) return rc;
    if ((rc = launch_pack_tables(op->view(), op->wsc, op->wss, op->wrc, op->wrs, op->stab, op->rtab, op->srng,
                                 op->rrng, nullptr)))
        return rc;
    if (!op->grng && (rc = dev_alloc(&op->grng, (size_t)((op->nr + 7) / 8) * ncol, "alloc receiver group ranges")))
        return rc;
    if ((rc = launch_group_ranges(op->rrng, op->grng, op->nr, ncol, nullptr))) return rc;
    op->stab_map_ok = make_record_map(&op->stab_map, op->stab, op->ni, op->ns, false) == KGB_OK;
    if (op->bf16_weights) {
        if (!op->stab2 && (rc = dev_alloc(&op->stab2, (size_t)op->ns * op->ni, "alloc bf16 source records"))) return rc;
        if (!op->rtab2 && (rc = dev_alloc(&op->rtab2, (size_t)op->nr * op->ni, "alloc bf16 receiver records")))
            return rc;
        if ((rc = launch_pack_tables_bf16(op->view(), op->wsc, op->wss, op->wrc, op->wrs, op->stab2, op->rtab2,
                                          nullptr)))
            return rc;
        op->stab2_map_ok = make_record_map(&op->stab2_map, op->stab2, op->ni, op->ns, true) == KGB_OK;
    }
    KGB_CUDA_TRY(cudaDeviceSynchronize());
    return KGB_OK;
}

// Offset aperture (kirchhoff.py:866-880): |six-rix|/(iz+1) < apmax, which
// holds from the first passing depth downwards; inside it the reference's
// taper index is 0 and taper[0] == 1, so only this cut-off acts.  Uploads
// the first passing depth per trace.
static int set_offset_gate(kgb_kirchhoff* op, double apmax, const int64_t* six, const int64_t* rix) {
    const int64_t npair = op->npair();
    std::vector<int32_t> izmin(npair);
    bool gate = false;
    for (int64_t p = 0; p < npair; ++p) {
        const double off = fabs((double)(six[p] - rix[p]));
        int iz = 0;
        while (iz < op->nz && !(off / (double)(iz + 1) < apmax)) ++iz;
        izmin[p] = iz;
        gate = gate || iz > 0;
    }
    int rc;
    if ((rc = dev_alloc(&op->izmin, izmin.size(), "alloc aperture"))) return rc;
    KGB_CUDA_TRY(cudaMemcpy(op->izmin, izmin.data(), izmin.size() * 4, cudaMemcpyHostToDevice));
    op->has_gate = gate;
    return KGB_OK;
}

// Whether the fixed-point spread may use split accumulation: count, once
// per table change, the most contributions any bin can receive, and keep
// the 64-bit accumulator of wide contributions (zeroed once; each forward
// leaves it zero) when that count is small enough.
static int update_split(kgb_kirchhoff* op) {
    op->split_ok = false;
    if (!op->trav_ready || (op->dynamic && !op->dyn_ready) || op->tq1) return KGB_OK;
    int rc;
    if (!op->count_buf && (rc = dev_alloc(&op->count_buf, 1, "alloc count word"))) return rc;
    if ((rc = launch_spread_count(op->view(), op->dynamic, op->has_gate, op->L, op->count_buf, nullptr))) return rc;
    unsigned count = 0u;
    KGB_CUDA_TRY(cudaMemcpy(&count, op->count_buf, sizeof(unsigned), cudaMemcpyDeviceToHost));
    op->max_bin_count = count;
    if (count > kSplitMaxCount) return KGB_OK;
    if (!op->wacc) {
        if ((rc = dev_alloc(&op->wacc, (size_t)op->ndata(), "alloc wide accumulator"))) return rc;
        KGB_CUDA_TRY(cudaMemset(op->wacc, 0, (size_t)op->ndata() * sizeof(unsigned long long)));
    }
    op->split_ok = true;
    return KGB_OK;
}

}  // namespace kgb

using namespace kgb;

extern "C" {

int kgb_version(void) { return 100; }

const char* kgb_last_error(void) { return g_last_error.c_str(); }

int kgb_kirchhoff_create(kgb_kirchhoff** out, int ns, int nr, int nt, int64_t ni, int nz, double dt,
                         int dynamic, const double* wav, int nwav, int wavcenter) {
    if (!out) return set_error(KGB_ERR_VALUE, "create: null output handle");
    *out = nullptr;
    if (ns <= 0 || nr <= 0 || nt < 2 || ni <= 0 || nz <= 0 || ni % nz != 0 || nz > 32767)
        return set_error(KGB_ERR_VALUE, "create: bad sizes ns=%d nr=%d nt=%d ni=%lld nz=%d", ns, nr, nt,
                         (long long)ni, nz);
    if (!(dt > 0.0) || !isfinite(dt)) return set_error(KGB_ERR_VALUE, "create: dt must be positive");
    if (!wav || nwav <= 0) return set_error(KGB_ERR_VALUE, "create: empty wavelet");
    if (wavcenter > nwav - 1 || wavcenter < 0)
        return set_error(KGB_ERR_VALUE, "offset must be smaller than h.shape[axis] - 1");
    if ((int64_t)ns * nr * (int64_t)nt > ((int64_t)1 << 40))
        return set_error(KGB_ERR_VALUE, "create: data volume too large");
    // filter padding of _Convolve1Dshort (convolve1d.py:76-88)
    int off = 2 * (nwav / 2 - wavcenter);
    if (nwav % 2 == 0) off -= 1;
    const int padl = std::max(off, 0), padr = -std::min(off, 0);
    std::vector<float> h(nwav + padl + padr, 0.f);
    for (int k = 0; k < nwav; ++k) h[padl + k] = (float)wav[k];
    std::vector<float> hf(h.rbegin(), h.rend());

    kgb_kirchhoff* op = new kgb_kirchhoff();
    op->ns = ns; op->nr = nr; op->nt = nt; op->ni = ni; op->nz = nz; op->dt = dt;
    op->dynamic = dynamic ? 1 : 0;
    op->L = (int)h.size();
    int rc = KGB_OK;
    cudaGetDevice(&op->device);
    do {
        if ((rc = dev_alloc(&op->h_dev, h.size(), "alloc wavelet"))) break;
        if ((rc = dev_alloc(&op->hflip_dev, h.size(), "alloc wavelet"))) break;
        cudaError_t e = cudaMemcpy(op->h_dev, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { rc = cuda_error(e, "upload wavelet"); break; }
        e = cudaMemcpy(op->hflip_dev, hf.data(), hf.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) { rc = cuda_error(e, "upload wavelet"); break; }
        if ((rc = dev_alloc(&op->tsq, (size_t)ns * ni, "alloc source traveltimes"))) break;
        if ((rc = dev_alloc(&op->trq, (size_t)nr * ni, "alloc receiver traveltimes"))) break;
        if ((rc = dev_alloc(&op->dcorr, (size_t)2 * op->ndata(), "alloc correlation scratch"))) break;
        op->partial_elems = gather_partial_elems(op->view());
        if ((rc = dev_alloc(&op->partial, (size_t)op->partial_elems, "alloc partial images"))) break;
        if ((rc = dev_alloc(&op->mv, (size_t)ni, "alloc scaled model"))) break;
        if ((rc = dev_alloc(&op->absmax, kScaleWords, "alloc forward scale block"))) break;
        if ((rc = dev_alloc(&op->err, 1, "alloc error word"))) break;
        e = cudaMemset(op->err, 0, sizeof(unsigned));
        if (e != cudaSuccess) { rc = cuda_error(e, "clear error word"); break; }
        if ((rc = prepare_kernels(op->view(), op->L))) break;
        if ((rc = static_scratch_prepare())) break;
        e = cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { rc = cuda_error(e, "create stream"); break; }
    } while (0);
    if (rc != KGB_OK) {
        kgb_kirchhoff_destroy(op);
        return rc;
    }
    *out = op;
    return KGB_OK;
}

int kgb_kirchhoff_destroy(kgb_kirchhoff* op) {
    if (!op) return KGB_OK;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(op->device);
    void* ptrs[] = {op->h_dev, op->hflip_dev, op->tsq, op->trq, op->wsc, op->wss, op->wrc, op->wrs,
                    op->vscale, op->izmin, op->dcorr, op->partial, op->m_stage, op->d_stage,
                    op->mv, op->absmax, op->stab, op->rtab, op->srng, op->rrng, op->tq1, op->tw1,
                    op->stab2, op->rtab2, op->grng, op->wacc, op->count_buf, op->err, op->trav64_s,
                    op->trav64_r, op->dist64_s, op->dist64_r, op->ang64_s, op->ang64_r};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (op->stream) cudaStreamDestroy(op->stream);
    if (op->stream2) cudaStreamDestroy(op->stream2);
    if (op->cstream) cudaStreamDestroy(op->cstream);
    for (cudaEvent_t e : op->ev)
        if (e) cudaEventDestroy(e);
    cudaSetDevice(dev);
    delete op;
    return KGB_OK;
}

int kgb_kirchhoff_set_traveltimes(kgb_kirchhoff* op, const double* ts, const double* tr) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (!ts || !tr) return set_error(KGB_ERR_VALUE, "set_traveltimes: null table");
    const int64_t ni = op->ni;
    const double inv_dt = 1.0 / op->dt;
    double maxs = 0.0, mins = INFINITY, minr = INFINITY;
    int64_t bad = -1;
    const int64_t n_s = ni * op->ns, n_r = ni * op->nr;
#pragma omp parallel for reduction(max : maxs) reduction(max : bad) reduction(min : mins) reduction(min : minr)
    for (int64_t k = 0; k < n_s + n_r; ++k) {
        const double t = (k < n_s ? ts[k] : tr[k - n_s]) * inv_dt;
        const double v = fabs(t);
        if (!isfinite(v)) bad = std::max(bad, k);
        else maxs = std::max(maxs, v);
        if (k < n_s) mins = std::min(mins, t);
        else minr = std::min(minr, t);
    }
    if (bad >= 0)
        return set_error(KGB_ERR_VALUE, "set_traveltimes: non-finite traveltime at flat index %lld", (long long)bad);
    const int F = choose_frac_bits(maxs, op->nt);
    if (F < 8)
        return set_error(KGB_ERR_VALUE, "set_traveltimes: traveltimes up to %.3g samples exceed the 32-bit fixed-point range", maxs);
    const double scale = ldexp(1.0, F);
    // transpose (ni, n) -> (n, ni) while quantising, in cache-sized blocks
    auto quantise = [&](const double* src, int n, std::vector<int32_t>& dst) {
        dst.resize((size_t)n * ni);
        const int64_t B = 64;
#pragma omp parallel for schedule(static)
        for (int64_t i0 = 0; i0 < ni; i0 += B)
            for (int j0 = 0; j0 < n; j0 += (int)B)
                for (int64_t i = i0; i < std::min(ni, i0 + B); ++i)
                    for (int j = j0; j < std::min(n, j0 + (int)B); ++j)
                        dst[(size_t)j * ni + i] = (int32_t)llrint(src[(size_t)i * n + j] * inv_dt * scale);
    };
    std::vector<int32_t> qs, qr;
    quantise(ts, op->ns, qs);
    quantise(tr, op->nr, qr);
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    KGB_CUDA_TRY(cudaMemcpy(op->tsq, qs.data(), qs.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    KGB_CUDA_TRY(cudaMemcpy(op->trq, qr.data(), qr.size() * sizeof(int32_t), cudaMemcpyHostToDevice));
    op->frac_bits = F;
    // every ts + tr >= 0 (after quantisation): the kernels may skip the
    // reference's negative-time case (-1 < t/dt < 0 -> it = 0, w < 0)
    int32_t qmin_s = INT32_MAX, qmin_r = INT32_MAX;
    for (int32_t q : qs) qmin_s = std::min(qmin_s, q);
    for (int32_t q : qr) qmin_r = std::min(qmin_r, q);
    op->nonneg = (int64_t)qmin_s + (int64_t)qmin_r >= 0;
    (void)mins; (void)minr;
    op->trav_ready = true;
    int rc = repack(op);
    return rc ? rc : update_split(op);
}

int kgb_kirchhoff_set_weight_precision(kgb_kirchhoff* op, int bf16) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (bf16 && !op->dynamic) return set_error(KGB_ERR_VALUE, "bf16 weights need a dynamic operator");
    if (bf16 != 0 && bf16 != 1) return set_error(KGB_ERR_VALUE, "weight precision: 0 (float32) or 1 (bf16)");
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    const bool was = op->bf16_weights;
    op->bf16_weights = bf16 == 1;
    if (op->bf16_weights && !was) {
        int rc = repack(op);  // builds the bf16 records if the tables are set
        if (rc) {
            op->bf16_weights = false;
            return rc;
        }
    }
    if (op->bf16_weights != was) return update_split(op);
    return KGB_OK;
}

int kgb_kirchhoff_set_traveltime_table(kgb_kirchhoff* op, const double* trav) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (!trav) return set_error(KGB_ERR_VALUE, "set_traveltime_table: null table");
    if (op->dynamic)
        return set_error(KGB_ERR_NOT_IMPLEMENTED,
                         "separate traveltime tables must be provided when selecting mode=dynamic");
    const int64_t ni = op->ni;
    const int nsnr = (int)op->npair();
    const int64_t n = ni * nsnr;
    const double inv_dt = 1.0 / op->dt;
    double maxs = 0.0, mins = INFINITY;
    int64_t bad = -1;
#pragma omp parallel for reduction(max : maxs) reduction(max : bad) reduction(min : mins)
    for (int64_t k = 0; k < n; ++k) {
        const double u = trav[k] * inv_dt;
        if (!isfinite(u)) bad = std::max(bad, k);
        else {
            maxs = std::max(maxs, fabs(u));
            mins = std::min(mins, u);
        }
    }
    if (bad >= 0)
        return set_error(KGB_ERR_VALUE, "set_traveltime_table: non-finite traveltime at flat index %lld",
                         (long long)bad);
    // fixed point (index exact, fraction to 2^-F) when every time is >= 0;
    // otherwise the truncated index and the fraction separately, which keeps
    // the reference's -1 < t/dt < 0 case (index 0, negative fraction)
    const bool fixed = mins >= 0.0;
    const int F = choose_frac_bits(std::min(maxs, (double)op->nt + 2.0), op->nt);
    const double scale = ldexp(1.0, F);
    const int64_t fmax = ((int64_t)1 << F) - 1;
    int rc;
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    if (!op->tq1 && (rc = dev_alloc(&op->tq1, (size_t)n, "alloc traveltime table"))) return rc;
    if (!fixed && !op->tw1 && (rc = dev_alloc(&op->tw1, (size_t)n, "alloc traveltime fractions"))) return rc;
    if (fixed && op->tw1) {
        cudaFree(op->tw1);
        op->tw1 = nullptr;
    }
    // (ni, nsnr) -> (nsnr, ni), a chunk of traces at a time
    const int C = (int)std::max<int64_t>(1, std::min<int64_t>(nsnr, (int64_t)(64 << 20) / std::max<int64_t>(ni, 1)));
    std::vector<int32_t> q((size_t)C * ni);
    std::vector<float> wv(fixed ? 0 : (size_t)C * ni);
    for (int j0 = 0; j0 < nsnr; j0 += C) {
        const int nj = std::min(C, nsnr - j0);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < ni; ++i) {
            const double* row = trav + (size_t)i * nsnr + j0;
            for (int j = 0; j < nj; ++j) {
                const double u = row[j] * inv_dt;
                // itrav = (trav / dt).astype(int32): truncation toward zero
                const double ut = std::max(-1073741824.0, std::min(1073741824.0, u));
                const int32_t it = (int32_t)ut;
                int32_t v;
                if (fixed) {
                    if (it >= op->nt) {
                        v = INT32_MAX;  // outside the trace: never valid
                    } else {
                        int64_t fq = llrint((u - it) * scale);
                        fq = std::max<int64_t>(0, std::min(fq, fmax));
                        v = (int32_t)(((int64_t)it << F) + fq);
                    }
                } else {
                    v = it;
                    wv[(size_t)j * ni + i] = (float)(u - it);
                }
                q[(size_t)j * ni + i] = v;
            }
        }
        KGB_CUDA_TRY(cudaMemcpy(op->tq1 + (size_t)j0 * ni, q.data(), (size_t)nj * ni * sizeof(int32_t),
                                cudaMemcpyHostToDevice));
        if (!fixed)
            KGB_CUDA_TRY(cudaMemcpy(op->tw1 + (size_t)j0 * ni, wv.data(), (size_t)nj * ni * sizeof(float),
                                    cudaMemcpyHostToDevice));
    }
    op->frac_bits = F;
    op->nonneg = true;
    op->trav_ready = true;
    return KGB_OK;
}

int kgb_kirchhoff_set_dynamic(kgb_kirchhoff* op, const double* amp_s, const double* amp_r,
                              const double* ang_s, const double* ang_r, const double* vel,
                              const double* aperture2, const double* angleaperture2,
                              const double* taper21, const int64_t* six, const int64_t* rix) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (!op->dynamic) return set_error(KGB_ERR_STATE, "set_dynamic: operator was created kinematic");
    if (!amp_s || !amp_r || !ang_s || !ang_r || !vel || !aperture2 || !angleaperture2 || !taper21 || !six || !rix)
        return set_error(KGB_ERR_VALUE, "set_dynamic: null table");
    if (taper21[0] != 1.0)
        return set_error(KGB_ERR_VALUE, "set_dynamic: aperture taper must start at 1 (taper(41, 20, 'hanning')[20:])");
    const int64_t ni = op->ni;
    const double amin = angleaperture2[0], amax = angleaperture2[1];
    const double dang = amax - amin;
    // angle taper of kirchhoff.py:845-864, folded per table entry; entries
    // outside the angle aperture get weight 0, which rejects the pair-point
    // exactly as the reference's `abs_angle < angleaperturemax` test does.
    auto fold = [&](const double* amp, const double* ang, int n, std::vector<float>& wc, std::vector<float>& ws) {
        wc.resize((size_t)n * ni);
        ws.resize((size_t)n * ni);
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < ni; ++i) {
            for (int j = 0; j < n; ++j) {
                const double a = ang[(size_t)i * n + j];
                const double A = amp[(size_t)i * n + j];
                const double aa = fabs(a);
                double tap = 0.0;
                if (aa < amax) {
                    tap = 1.0;
                    if (aa >= amin) {
                        double q = py_floordiv(20.0 * (aa - amin), dang);
                        long idx = (long)q;
                        if (idx < 0) idx = 0;
                        if (idx > 20) idx = 20;
                        tap = taper21[idx];
                    }
                }
                const double base = A * tap;
                wc[(size_t)j * ni + i] = (float)(base * cos(a / 2.0));
                ws[(size_t)j * ni + i] = (float)(base * sin(a / 2.0));
            }
        }
    };
    std::vector<float> wsc, wss, wrc, wrs;
    fold(amp_s, ang_s, op->ns, wsc, wss);
    fold(amp_r, ang_r, op->nr, wrc, wrs);
    std::vector<float> vs(ni);
    for (int64_t i = 0; i < ni; ++i) vs[i] = (float)(2.0 / vel[i]);
    // |wc_s wc_r + ws_s ws_r| <= |A_s tap_s| |A_r tap_r| (Cauchy-Schwarz): the
    // bound the forward's fixed-point scale uses
    auto maxabs2 = [](const std::vector<float>& c, const std::vector<float>& s_) {
        double m = 0.0;
        for (size_t k = 0; k < c.size(); ++k) m = std::max(m, sqrt((double)c[k] * c[k] + (double)s_[k] * s_[k]));
        return m;
    };
    const double wmax = maxabs2(wsc, wss) * maxabs2(wrc, wrs) * 1.0001;
    if (!isfinite(wmax)) return set_error(KGB_ERR_VALUE, "set_dynamic: non-finite amplitude or angle table");
    // offset aperture (kirchhoff.py:866-880): |six-rix|/(iz+1) < apmax, which
    // holds from the first passing depth downwards; inside it the reference's
    // taper index is 0 and taper[0] == 1, so only this cut-off acts.
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    int rc;
    if ((rc = dev_alloc(&op->wsc, wsc.size(), "alloc weights"))) return rc;
    if ((rc = dev_alloc(&op->wss, wss.size(), "alloc weights"))) return rc;
    if ((rc = dev_alloc(&op->wrc, wrc.size(), "alloc weights"))) return rc;
    if ((rc = dev_alloc(&op->wrs, wrs.size(), "alloc weights"))) return rc;
    if ((rc = dev_alloc(&op->vscale, vs.size(), "alloc velocity"))) return rc;
    KGB_CUDA_TRY(cudaMemcpy(op->wsc, wsc.data(), wsc.size() * 4, cudaMemcpyHostToDevice));
    KGB_CUDA_TRY(cudaMemcpy(op->wss, wss.data(), wss.size() * 4, cudaMemcpyHostToDevice));
    KGB_CUDA_TRY(cudaMemcpy(op->wrc, wrc.data(), wrc.size() * 4, cudaMemcpyHostToDevice));
    KGB_CUDA_TRY(cudaMemcpy(op->wrs, wrs.data(), wrs.size() * 4, cudaMemcpyHostToDevice));
    KGB_CUDA_TRY(cudaMemcpy(op->vscale, vs.data(), vs.size() * 4, cudaMemcpyHostToDevice));
    if ((rc = set_offset_gate(op, aperture2[1], six, rix))) return rc;
    op->wmax = (float)std::max(wmax, 1e-30);
    op->dyn_ready = true;
    rc = repack(op);
    return rc ? rc : update_split(op);
}

static int check_ready(const kgb_kirchhoff* op) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (!op->trav_ready) return set_error(KGB_ERR_STATE, "traveltime tables not set");
    if (op->dynamic && !op->dyn_ready) return set_error(KGB_ERR_STATE, "dynamic tables not set");
    return KGB_OK;
}

int kgb_kirchhoff_spread(kgb_kirchhoff* op, const float* m, float* d, void* stream) {
    int rc = check_ready(op);
    if (rc) return rc;
    if (!m || !d) return set_error(KGB_ERR_VALUE, "spread: null pointer");
    return launch_spread(op->view(), op->dynamic, op->has_gate, m, d, nullptr, 0, false, (cudaStream_t)stream);
}

int kgb_kirchhoff_forward(kgb_kirchhoff* op, const float* m, float* d, void* stream) {
    int rc = check_ready(op);
    if (rc) return rc;
    if (!m || !d) return set_error(KGB_ERR_VALUE, "forward: null pointer");
    return launch_spread(op->view(), op->dynamic, op->has_gate, m, d, op->h_dev, op->L, true, (cudaStream_t)stream);
}

int kgb_kirchhoff_gather(kgb_kirchhoff* op, const float* d, float* m, void* stream) {
    int rc = check_ready(op);
    if (rc) return rc;
    if (!m || !d) return set_error(KGB_ERR_VALUE, "gather: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = launch_wavelet(d, op->dcorr, op->npair(), op->nt, nullptr, 1, 1, s))) return rc;
    return launch_gather(op->view(), op->dynamic, op->has_gate, op->dcorr, m, op->partial, op->partial_elems, s);
}

int kgb_kirchhoff_adjoint(kgb_kirchhoff* op, const float* d, float* m, void* stream) {
    int rc = check_ready(op);
    if (rc) return rc;
    if (!m || !d) return set_error(KGB_ERR_VALUE, "adjoint: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = launch_wavelet(d, op->dcorr, op->npair(), op->nt, op->hflip_dev, op->L, 1, s))) return rc;
    return launch_gather(op->view(), op->dynamic, op->has_gate, op->dcorr, m, op->partial, op->partial_elems, s);
}

int kgb_kirchhoff_wavelet(kgb_kirchhoff* op, const float* x, float* y, int adjoint, void* stream) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (!x || !y) return set_error(KGB_ERR_VALUE, "wavelet: null pointer");
    return launch_wavelet(x, y, op->npair(), op->nt, adjoint ? op->hflip_dev : op->h_dev, op->L, 0,
                          (cudaStream_t)stream);
}

static int ensure_stage(kgb_kirchhoff* op) {
    int rc;
    if (!op->m_stage && (rc = dev_alloc(&op->m_stage, (size_t)op->ni, "alloc model staging"))) return rc;
    if (!op->d_stage && (rc = dev_alloc(&op->d_stage, (size_t)op->ndata(), "alloc data staging"))) return rc;
    return KGB_OK;
}

static int ensure_streams(kgb_kirchhoff* op) {
    if (!op->stream2) KGB_CUDA_TRY(cudaStreamCreateWithFlags(&op->stream2, cudaStreamNonBlocking));
    if (!op->cstream) KGB_CUDA_TRY(cudaStreamCreateWithFlags(&op->cstream, cudaStreamNonBlocking));
    for (cudaEvent_t& e : op->ev)
        if (!e) KGB_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return KGB_OK;
}

// Forward with host buffers.  With the fixed-point spread the receiver
// groups run as kHostChunks launches alternating between two streams (a
// launch fills the tail of the previous one) and each chunk's traces go to
// the host on a copy stream while the next chunks compute.  Every trace is
// computed exactly as in one launch.
int kgb_kirchhoff_forward_host(kgb_kirchhoff* op, const float* m_host, float* d_host) {
    int rc = check_ready(op);
    if (rc) return rc;
    if (!m_host || !d_host) return set_error(KGB_ERR_VALUE, "forward_host: null pointer");
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    if ((rc = ensure_stage(op))) return rc;
    cudaStream_t s = op->stream;
    KGB_CUDA_TRY(cudaMemcpyAsync(op->m_stage, m_host, (size_t)op->ni * 4, cudaMemcpyHostToDevice, s));
    kgb::KirchDev K = op->view();
    const int R = spread_group_size(K, op->L);
    const size_t pitch = (size_t)op->nr * op->nt * 4;
    if (R == 0 || pitch > ((size_t)1 << 30)) {
        if ((rc = kgb_kirchhoff_forward(op, op->m_stage, op->d_stage, s))) return rc;
        KGB_CUDA_TRY(cudaMemcpyAsync(d_host, op->d_stage, (size_t)op->ndata() * 4, cudaMemcpyDeviceToHost, s));
        KGB_CUDA_TRY(cudaStreamSynchronize(s));
        return KGB_OK;
    }
    if ((rc = ensure_streams(op))) return rc;
    if ((rc = launch_spread_prepass(K, op->dynamic, op->m_stage, s))) return rc;
    KGB_CUDA_TRY(cudaEventRecord(op->ev[0], s));
    KGB_CUDA_TRY(cudaStreamWaitEvent(op->stream2, op->ev[0], 0));
    const int ngroups = (op->nr + R - 1) / R;
    const int nch = std::min(kgb_kirchhoff::kHostChunks, ngroups);
    K.prepass = 0;
    for (int c = 0; c < nch; ++c) {
        K.g0 = (int)((int64_t)c * ngroups / nch);
        K.g1 = (int)((int64_t)(c + 1) * ngroups / nch);
        cudaStream_t sc = (c & 1) ? op->stream2 : s;
        if ((rc = launch_spread(K, op->dynamic, op->has_gate, op->m_stage, op->d_stage, op->h_dev, op->L, true, sc)))
            return rc;
        KGB_CUDA_TRY(cudaEventRecord(op->ev[1 + c], sc));
        KGB_CUDA_TRY(cudaStreamWaitEvent(op->cstream, op->ev[1 + c], 0));
        const int r_lo = K.g0 * R, r_hi = std::min(op->nr, K.g1 * R);
        const size_t off = (size_t)r_lo * op->nt;
        KGB_CUDA_TRY(cudaMemcpy2DAsync(d_host + off, pitch, op->d_stage + off, pitch, (size_t)(r_hi - r_lo) * op->nt * 4,
                                       (size_t)op->ns, cudaMemcpyDeviceToHost, op->cstream));
    }
    KGB_CUDA_TRY(cudaStreamSynchronize(op->cstream));
    return KGB_OK;
}

// Adjoint with host buffers: the data go to the device in kHostChunks
// source blocks on a copy stream and each block is correlated with the
// wavelet as soon as it lands; the gather runs once all are in.
int kgb_kirchhoff_adjoint_host(kgb_kirchhoff* op, const float* d_host, float* m_host) {
    int rc = check_ready(op);
    if (rc) return rc;
    if (!m_host || !d_host) return set_error(KGB_ERR_VALUE, "adjoint_host: null pointer");
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    if ((rc = ensure_stage(op)) || (rc = ensure_streams(op))) return rc;
    cudaStream_t s = op->stream;
    // the copy stream may only overwrite the staging buffer after the
    // previous work on it is done
    KGB_CUDA_TRY(cudaEventRecord(op->ev[0], s));
    KGB_CUDA_TRY(cudaStreamWaitEvent(op->cstream, op->ev[0], 0));
    const int nch = std::min(kgb_kirchhoff::kHostChunks, op->ns);
    for (int c = 0; c < nch; ++c) {
        const int s0 = (int)((int64_t)c * op->ns / nch), s1 = (int)((int64_t)(c + 1) * op->ns / nch);
        const size_t off = (size_t)s0 * op->nr * op->nt;
        const int64_t ntr = (int64_t)(s1 - s0) * op->nr;
        KGB_CUDA_TRY(cudaMemcpyAsync(op->d_stage + off, d_host + off, (size_t)ntr * op->nt * 4, cudaMemcpyHostToDevice,
                                     op->cstream));
        KGB_CUDA_TRY(cudaEventRecord(op->ev[1 + c], op->cstream));
        KGB_CUDA_TRY(cudaStreamWaitEvent(s, op->ev[1 + c], 0));
        if ((rc = launch_wavelet(op->d_stage + off, op->dcorr + 2 * off, ntr, op->nt, op->hflip_dev, op->L, 1, s)))
            return rc;
    }
    if ((rc = launch_gather(op->view(), op->dynamic, op->has_gate, op->dcorr, op->m_stage, op->partial,
                            op->partial_elems, s)))
        return rc;
    KGB_CUDA_TRY(cudaMemcpyAsync(m_host, op->m_stage, (size_t)op->ni * 4, cudaMemcpyDeviceToHost, s));
    KGB_CUDA_TRY(cudaStreamSynchronize(s));
    return KGB_OK;
}

int kgb_kirchhoff_set_variant(kgb_kirchhoff* op, int spread_variant) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (spread_variant < 0 || spread_variant > 3)
        return set_error(KGB_ERR_VALUE, "set_variant: spread variant must be 0, 1, 2 or 3");
    op->spread_variant = spread_variant;
    return KGB_OK;
}

int kgb_kirchhoff_set_adjoint_variant(kgb_kirchhoff* op, int variant) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (variant < 0 || variant > 2) return set_error(KGB_ERR_VALUE, "adjoint variant: 0, 1 or 2");
    op->adjoint_variant = variant;
    return KGB_OK;
}

int kgb_kirchhoff_info(const kgb_kirchhoff* op, int64_t* s) {
    if (!op || !s) return set_error(KGB_ERR_VALUE, "info: null pointer");
    for (int k = 0; k < 16; ++k) s[k] = 0;
    s[0] = op->ns; s[1] = op->nr; s[2] = op->nt; s[3] = op->ni;
    s[4] = op->frac_bits; s[5] = op->L; s[6] = op->has_gate ? 1 : 0; s[7] = op->dynamic;
    s[8] = op->nonneg ? 1 : 0;
    s[9] = gather_nsplit(op->view(), op->dynamic, op->has_gate);
    // kernels per application: forward = prepass + scale choice + spread;
    // adjoint = correlation + gather (+ partial-image sum when split)
    s[10] = 3;
    s[11] = 2 + (s[9] > 1 ? 1 : 0);
    s[12] = op->spread_variant;
    s[13] = op->split_ok ? 1 : 0;
    s[14] = op->max_bin_count;
    // staged adjoint in use, and the error word of the bounded waits
    unsigned err = 0u;
    if (op->err && cudaMemcpy(&err, op->err, sizeof(unsigned), cudaMemcpyDeviceToHost) != cudaSuccess)
        return set_error(KGB_ERR_CUDA, "info: reading the error word failed");
    const kgb::KirchDev K = op->view();
    const int used = !op->dynamic ? 0 : K.rec_map ? 2 : (K.adjoint_variant == 1 && K.ns <= 64 && K.srng) ? 1 : 0;
    s[15] = used | ((int64_t)err << 2);
    return KGB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Tables built on the device (tables.cu)
// ---------------------------------------------------------------------------
namespace {

template <typename T>
struct DevBuf {  // scratch freed on every return path
    T* p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
};

template <typename T>
int upload(DevBuf<T>& b, const T* host, size_t n, const char* what) {
    int rc = dev_alloc(&b.p, n, what);
    if (rc) return rc;
    KGB_CUDA_TRY(cudaMemcpy(b.p, host, n * sizeof(T), cudaMemcpyHostToDevice));
    return KGB_OK;
}

double read_absmax(const unsigned long long* dev) {
    unsigned long long bits = 0;
    cudaMemcpy(&bits, dev, sizeof(bits), cudaMemcpyDeviceToHost);
    double v;
    memcpy(&v, &bits, sizeof(v));
    return v;
}

}  // namespace

int kgb_kirchhoff_build_tables(kgb_kirchhoff* op, int mode, int ndim, const double* yax, int ny, const double* xax,
                               int nx, const double* zax, int nz, const double* srcs, const double* recs,
                               const double* vel, int64_t nvel, const double* aperture2,
                               const double* angleaperture2, const double* taper21, const int64_t* six,
                               const int64_t* rix, double* maxdist_out) {
    if (!op) return set_error(KGB_ERR_STATE, "null operator");
    if (mode != 0 && mode != 1) return set_error(KGB_ERR_VALUE, "build_tables: mode must be 0 (analytic) or 1 (eikonal)");
    if (ndim != 2 && ndim != 3) return set_error(KGB_ERR_VALUE, "build_tables: ndim must be 2 or 3");
    if (ndim == 2) ny = 1;
    if (!xax || !zax || (ndim == 3 && !yax) || !srcs || !recs || !vel)
        return set_error(KGB_ERR_VALUE, "build_tables: null argument");
    if (nx < 1 || nz < 1 || ny < 1 || (int64_t)ny * nx * nz != op->ni || nz != op->nz)
        return set_error(KGB_ERR_VALUE, "build_tables: grid %d x %d x %d does not match the operator", ny, nx, nz);
    if (mode == 0 && nvel != 1) return set_error(KGB_ERR_VALUE, "vel must be scalar for mode=analytical");
    if (mode == 1 && nvel != op->ni && nvel != 1) return set_error(KGB_ERR_VALUE, "build_tables: velocity size");
    if (nvel != 1 && nvel != op->ni) return set_error(KGB_ERR_VALUE, "build_tables: velocity size");
    for (int64_t k = 0; k < nvel; ++k)
        if (!(vel[k] > 0.0) || !isfinite(vel[k]))
            return set_error(KGB_ERR_VALUE, "build_tables: velocity must be positive and finite");
    if (op->dynamic && (!aperture2 || !angleaperture2 || !taper21 || !six || !rix))
        return set_error(KGB_ERR_VALUE, "build_tables: dynamic operator needs apertures, taper and six/rix");
    if (op->dynamic && taper21[0] != 1.0)
        return set_error(KGB_ERR_VALUE, "build_tables: aperture taper must start at 1 (taper(41, 20, 'hanning')[20:])");
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    const int ns = op->ns, nr = op->nr;
    const int64_t ni = op->ni;
    TableGeom g;
    g.ndim = ndim;
    g.ny = ny;
    g.nx = nx;
    g.nz = nz;
    g.ni = ni;
    g.hy = ndim == 3 && ny > 1 ? yax[1] - yax[0] : 1.0;
    g.hx = nx > 1 ? xax[1] - xax[0] : 1.0;
    g.hz = nz > 1 ? zax[1] - zax[0] : 1.0;
    int rc;
    if ((rc = dev_alloc(&op->trav64_s, (size_t)ns * ni, "alloc source traveltime rows"))) return rc;
    if ((rc = dev_alloc(&op->trav64_r, (size_t)nr * ni, "alloc receiver traveltime rows"))) return rc;
    if ((rc = dev_alloc(&op->dist64_s, (size_t)ns * ni, "alloc source distance rows"))) return rc;
    if ((rc = dev_alloc(&op->dist64_r, (size_t)nr * ni, "alloc receiver distance rows"))) return rc;
    if (mode == 0) {
        DevBuf<double> dy, dx, dz, ps, pr;
        if (ndim == 3 && (rc = upload(dy, yax, ny, "upload y axis"))) return rc;
        if ((rc = upload(dx, xax, nx, "upload x axis"))) return rc;
        if ((rc = upload(dz, zax, nz, "upload z axis"))) return rc;
        if ((rc = upload(ps, srcs, (size_t)ndim * ns, "upload sources"))) return rc;
        if ((rc = upload(pr, recs, (size_t)ndim * nr, "upload receivers"))) return rc;
        if ((rc = launch_analytic_rows(g, dy.p, dx.p, dz.p, ps.p, ns, vel[0], op->trav64_s, op->dist64_s, nullptr)))
            return rc;
        if ((rc = launch_analytic_rows(g, dy.p, dx.p, dz.p, pr.p, nr, vel[0], op->trav64_r, op->dist64_r, nullptr)))
            return rc;
    } else {
        // grid coordinates of the points, sources then receivers:
        // round((p - origin) / spacing) (kirchhoff.py:615, 627); (x, z) in
        // 2-D, (y, x, z) in 3-D
        const int nd = ndim;
        std::vector<int> pts((size_t)nd * ((size_t)ns + nr));
        auto coords = [&](const double* p, int np, int* out) {
            for (int k = 0; k < np; ++k) {
                const double cx = nearbyint((p[(nd - 2) * (size_t)np + k] - xax[0]) / g.hx);
                const double cz = nearbyint((p[(nd - 1) * (size_t)np + k] - zax[0]) / g.hz);
                const double cy = nd == 3 ? nearbyint((p[k] - yax[0]) / g.hy) : 0.0;
                if (!(cx >= 0 && cx < nx && cz >= 0 && cz < nz && cy >= 0 && cy < ny)) return false;
                int* o = out + (size_t)nd * k;
                if (nd == 3) *o++ = (int)cy;
                o[0] = (int)cx;
                o[1] = (int)cz;
            }
            return true;
        };
        if (!coords(srcs, ns, pts.data()) || !coords(recs, nr, pts.data() + (size_t)nd * ns))
            return set_error(KGB_ERR_VALUE, "build_tables: a source or receiver lies outside the grid");
        DevBuf<int> dp;
        DevBuf<double> sp, corner;
        DevBuf<float> rhs;
        if ((rc = upload(dp, pts.data(), pts.size(), "upload table points"))) return rc;
        std::vector<double> vfull;
        const double* vp = vel;
        if (nvel == 1) {
            vfull.assign((size_t)ni, vel[0]);
            vp = vfull.data();
        }
        if ((rc = upload(sp, vp, (size_t)ni, "upload velocity"))) return rc;
        if ((rc = dev_alloc(&rhs.p, (size_t)ni, "alloc eikonal right-hand side"))) return rc;
        if ((rc = dev_alloc(&corner.p, (size_t)ni, "alloc corner distance table"))) return rc;
        KGB_CUDA_TRY(cudaMemset(op->err, 0, sizeof(unsigned)));
        if ((rc = launch_eikonal_tables(g, sp.p, rhs.p, dp.p, ns, nr, op->trav64_s, op->trav64_r, corner.p, op->err,
                                        nullptr)))
            return rc;
        if ((rc = launch_distance_rows(g, corner.p, dp.p, ns, nr, op->dist64_s, op->dist64_r, nullptr))) return rc;
        unsigned err = 0;
        KGB_CUDA_TRY(cudaMemcpy(&err, op->err, sizeof(unsigned), cudaMemcpyDeviceToHost));
        if (err) return set_error(KGB_ERR_CUDA, "build_tables: the eikonal sweeps did not converge");
    }
    // fixed-point traveltimes (the quantisation of kgb_kirchhoff_set_traveltimes)
    DevBuf<unsigned long long> red;
    if ((rc = dev_alloc(&red.p, 4, "alloc reduction words"))) return rc;
    DevBuf<long long> bad;
    if ((rc = dev_alloc(&bad.p, 1, "alloc check word"))) return rc;
    KGB_CUDA_TRY(cudaMemset(red.p, 0, 4 * sizeof(unsigned long long)));
    KGB_CUDA_TRY(cudaMemset(bad.p, 0xff, sizeof(long long)));
    if ((rc = launch_finite_check(op->trav64_s, (int64_t)ns * ni, bad.p, nullptr))) return rc;
    if ((rc = launch_finite_check(op->trav64_r, (int64_t)nr * ni, bad.p, nullptr))) return rc;
    if ((rc = launch_absmax(op->trav64_s, (int64_t)ns * ni, red.p, nullptr))) return rc;
    if ((rc = launch_absmax(op->trav64_r, (int64_t)nr * ni, red.p, nullptr))) return rc;
    long long badk = -1;
    KGB_CUDA_TRY(cudaMemcpy(&badk, bad.p, sizeof(badk), cudaMemcpyDeviceToHost));
    if (badk >= 0) return set_error(KGB_ERR_VALUE, "build_tables: non-finite traveltime");
    const double inv_dt = 1.0 / op->dt;
    const double maxs = read_absmax(red.p) * inv_dt;
    const int F = choose_frac_bits(maxs, op->nt);
    if (F < 8)
        return set_error(KGB_ERR_VALUE, "build_tables: traveltimes up to %.3g samples exceed the 32-bit fixed-point range",
                         maxs);
    DevBuf<int> qmin;
    if ((rc = dev_alloc(&qmin.p, 2, "alloc check word"))) return rc;
    const int big[2] = {INT32_MAX, INT32_MAX};
    KGB_CUDA_TRY(cudaMemcpy(qmin.p, big, sizeof(big), cudaMemcpyHostToDevice));
    const double scale = ldexp(1.0, F);
    if ((rc = launch_quantise(op->trav64_s, (int64_t)ns * ni, inv_dt, scale, op->tsq, qmin.p, nullptr))) return rc;
    if ((rc = launch_quantise(op->trav64_r, (int64_t)nr * ni, inv_dt, scale, op->trq, qmin.p + 1, nullptr))) return rc;
    int qm[2];
    KGB_CUDA_TRY(cudaMemcpy(qm, qmin.p, sizeof(qm), cudaMemcpyDeviceToHost));
    op->frac_bits = F;
    op->nonneg = (int64_t)qm[0] + (int64_t)qm[1] >= 0;
    op->trav_ready = true;
    op->table_ndim = ndim;
    // distances and amplitudes (kirchhoff.py:316-330)
    if ((rc = launch_absmax(op->dist64_s, (int64_t)ns * ni, red.p + 1, nullptr))) return rc;
    if ((rc = launch_absmax(op->dist64_r, (int64_t)nr * ni, red.p + 2, nullptr))) return rc;
    op->maxdist = 1e-2 * (read_absmax(red.p + 1) + read_absmax(red.p + 2));
    if (maxdist_out) *maxdist_out = op->maxdist;
    if (op->dynamic) {
        if ((rc = dev_alloc(&op->ang64_s, (size_t)ns * ni, "alloc source angle rows"))) return rc;
        if ((rc = dev_alloc(&op->ang64_r, (size_t)nr * ni, "alloc receiver angle rows"))) return rc;
        if ((rc = launch_angle_rows(g, op->trav64_s, nullptr, ns, op->ang64_s, nullptr))) return rc;
        // 3-D receivers: the x-gradient sign of the source row of the same
        // index when ns == nr (kirchhoff.py:386-393), else their own
        if ((rc = launch_angle_rows(g, op->trav64_r, (ndim == 3 && ns == nr) ? op->trav64_s : nullptr, nr,
                                    op->ang64_r, nullptr)))
            return rc;
        DevBuf<double> tap;
        if ((rc = upload(tap, taper21, 21, "upload taper"))) return rc;
        if ((rc = dev_alloc(&op->wsc, (size_t)ns * ni, "alloc weights"))) return rc;
        if ((rc = dev_alloc(&op->wss, (size_t)ns * ni, "alloc weights"))) return rc;
        if ((rc = dev_alloc(&op->wrc, (size_t)nr * ni, "alloc weights"))) return rc;
        if ((rc = dev_alloc(&op->wrs, (size_t)nr * ni, "alloc weights"))) return rc;
        KGB_CUDA_TRY(cudaMemset(red.p, 0, 2 * sizeof(unsigned long long)));
        const double amin = angleaperture2[0], amax = angleaperture2[1];
        if ((rc = launch_fold_rows(ndim, op->maxdist, amin, amax, tap.p, op->dist64_s, op->ang64_s, (int64_t)ns * ni,
                                   op->wsc, op->wss, red.p, nullptr)))
            return rc;
        if ((rc = launch_fold_rows(ndim, op->maxdist, amin, amax, tap.p, op->dist64_r, op->ang64_r, (int64_t)nr * ni,
                                   op->wrc, op->wrs, red.p + 1, nullptr)))
            return rc;
        const double wmax = read_absmax(red.p) * read_absmax(red.p + 1) * 1.0001;
        if (!isfinite(wmax)) return set_error(KGB_ERR_VALUE, "build_tables: non-finite amplitude or angle table");
        if ((rc = dev_alloc(&op->vscale, (size_t)ni, "alloc velocity"))) return rc;
        DevBuf<double> dv;
        if ((rc = upload(dv, vel, (size_t)nvel, "upload velocity"))) return rc;
        if ((rc = launch_vscale(dv.p, nvel, ni, op->vscale, nullptr))) return rc;
        if ((rc = set_offset_gate(op, aperture2[1], six, rix))) return rc;
        op->wmax = (float)std::max(wmax, 1e-30);
        op->dyn_ready = true;
    }
    KGB_CUDA_TRY(cudaDeviceSynchronize());
    rc = repack(op);
    return rc ? rc : update_split(op);
}

int kgb_kirchhoff_get_table(kgb_kirchhoff* op, int which, double* out_host) {
    if (!op || !out_host) return set_error(KGB_ERR_VALUE, "get_table: null argument");
    if (which < 0 || which > 5) return set_error(KGB_ERR_VALUE, "get_table: which must be 0..5");
    const bool src = which % 2 == 0;
    const int n = src ? op->ns : op->nr;
    const double* rows = nullptr;
    if (which < 2) rows = src ? op->trav64_s : op->trav64_r;
    else if (which < 4) rows = src ? op->dist64_s : op->dist64_r;
    else rows = src ? op->ang64_s : op->ang64_r;
    if (!rows) return set_error(KGB_ERR_STATE, "get_table: the table was not built on the device");
    KGB_CUDA_TRY(cudaSetDevice(op->device));
    const size_t cnt = (size_t)n * op->ni;
    DevBuf<double> tmp, amp;
    int rc;
    if (which == 2 || which == 3) {
        // amplitudes from the distance rows (kirchhoff.py:316-330)
        if ((rc = dev_alloc(&amp.p, cnt, "alloc amplitude rows"))) return rc;
        if ((rc = launch_amplitude_rows(rows, (int64_t)cnt, op->maxdist, op->table_ndim, amp.p, nullptr))) return rc;
        rows = amp.p;
    }
    if ((rc = dev_alloc(&tmp.p, cnt, "alloc table transpose"))) return rc;
    if ((rc = launch_rows_to_reference(rows, n, op->ni, tmp.p, nullptr))) return rc;
    KGB_CUDA_TRY(cudaMemcpy(out_host, tmp.p, cnt * sizeof(double), cudaMemcpyDeviceToHost));
    return KGB_OK;
}
