// Internal declarations shared by the CUDA translation units of
// libpylops_gb300.so.  Not part of the public C ABI (include/kirchhoff_gb300.h).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/kirchhoff_gb300.h"

namespace kgb {

// Record the failure message for kgb_last_error() and return `code`.
int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

#define KGB_CUDA_TRY(call)                                   \
    do {                                                     \
        cudaError_t _e = (call);                             \
        if (_e != cudaSuccess) return ::kgb::cuda_error(_e, #call); \
    } while (0)

// Device view of one operator's tables, passed by value to the kernels.
//
// Layout in HBM (all source-/receiver-major so that a warp's 32 consecutive
// image points read 128 contiguous bytes of one row):
//   tsq[is][ii], trq[ir][ii]   int32  traveltime in samples, fixed point with
//                                     frac_bits fractional bits
//   wsc/wss[is][ii]            f32    A_s * tap_s * cos(a_s/2), ... * sin(a_s/2)
//   wrc/wrs[ir][ii]            f32    same for receivers
//   vscale[ii]                 f32    2 / v(ii)
//   izmin[is*nr+ir]            int32  first depth index inside the offset aperture
struct KirchDev {
    int ns, nr, nt, nz;
    int64_t ni;
    int frac_bits;
    int nonneg;        // every ts + tr >= 0: index math without the negative-time case
    float wmax;        // bound on |dynamic weight| (1 for kinematic), for the fixed-point scale
    int spread_variant; // 0: fixed-point shared-memory atomics (the default); 1/2: warp-binned, 1/2 traces per warp;
                        // 3: fixed-point with the carry accumulation only
    float* mv;         // scratch: m * 2/v per application (ni)
    unsigned* absmax;  // scratch: the forward's scale block (kScaleWords, see fixed_acc.cuh) per application
    const int32_t* tsq;
    const int32_t* trq;
    const float* wsc;
    const float* wss;
    const float* wrc;
    const float* wrs;
    const float* vscale;
    const int32_t* izmin;
    // dynamic mode: per-entry records {tq, wc, ws, 0} (one 16-byte load gives
    // a table entry's traveltime and both weights)
    const int4* stab;  // [ns][ni]
    const int4* rtab;  // [nr][ni]
    // dynamic mode: per (row, depth column) the depth range [lo, hi) outside
    // which the row's weight is exactly zero, packed lo | hi << 16
    const uint32_t* srng;  // [ns][ncol]
    const uint32_t* rrng;  // [nr][ncol]
    // union of the ranges of each group of 8 consecutive receivers, packed
    // the same way: a point outside it has zero weight for all 8
    const uint32_t* grng;  // [ceil(nr/8)][ncol]
    // single traveltime table (one entry per image point and trace, mode
    // 'byot' with trav of shape (ni, ns*nr)): tq1[tr][ii] is the fixed-point
    // sample count (tw1 == nullptr) or, for tables with negative times, the
    // truncated index int(t/dt) with the fraction in tw1[tr][ii]
    const int32_t* tq1;
    const float* tw1;
    // dynamic mode with bf16 weights: 8-byte records {tq, bf16 wc | bf16 ws << 16}
    // used instead of stab/rtab when non-null
    const int2* stab2;  // [ns][ni]
    const int2* rtab2;  // [nr][ni]
    // fixed-point spread (variant 0) only: receiver groups [g0, g1) of this
    // launch, and whether it first computes mv and absmax (prepass = 0 when
    // an earlier launch on an ordered stream already did)
    int g0, g1;
    int prepass;
    // fixed-point spread: split accumulation (two fire-and-forget shared
    // atomics per contribution) when every bin of the operator receives at
    // most kSplitMaxCount contributions (split_ok, counted when the tables
    // were set) and the 64-bit accumulator of wide contributions wacc
    // ([ns*nr][nt], zero between applications) exists
    int split_ok;
    unsigned long long* wacc;
    unsigned* count_out;  // spread_count: the largest contribution count of any bin
    // adjoint: a TMA tensor map over the source records in use (stab, or
    // stab2 with bf16 weights) -- a HOST pointer, read by the launcher and
    // passed to the kernel by value; null: the gather loads records itself
    const CUtensorMap* rec_map;
    unsigned* err;  // device word: nonzero after a bounded wait of a kernel gave up
    // adjoint kernel of dynamic operators: 0 loads each source record in the
    // gather, 1 keeps the next active source's record in flight (at most 64
    // sources), 2 stages the records by TMA (rec_map); all give the same image
    int adjoint_variant;
};

// u32 words of the forward's fixed-point scale block: [0] bits of max |mv|,
// [1] the chosen scale exponent, [2, 2 + 256) histogram of the exponents of
// the nonzero |mv|
constexpr int kScaleWords = 2 + 256;

// Launchers (kirchhoff_kernels.cu).  All asynchronous on `stream`.
int launch_spread(const KirchDev& K, bool dynamic, bool gate, const float* m, float* y,
                  const float* h, int L, bool fuse_wavelet, cudaStream_t stream);
int launch_gather(const KirchDev& K, bool dynamic, bool gate, const float* d, float* img,
                  float* partial, int64_t partial_capacity, cudaStream_t stream);
// TMA tensor map over dynamic-mode source records ([ns][ni] int4, or int2
// with bf16 weights) for the staged adjoint; KGB_ERR_NOT_IMPLEMENTED when
// the layout does not allow one (the gather then loads records itself).
int make_record_map(CUtensorMap* map, const void* records, int64_t ni, int ns, bool half);
// Set the kernels' shared-memory attributes once, outside any stream capture.
int prepare_kernels(const KirchDev& K, int L);
// Wavelet filter along time.  interleave = 0 writes y[tr][n]; interleave = 1
// writes the pair (o[n], o[n+1]) at y[tr][2n] (o[nt] = 0), the layout the
// gather reads with one 8-byte load.  g == nullptr copies (no filter).
int launch_wavelet(const float* x, float* y, int64_t ntr, int nt, const float* g, int L,
                   int interleave, cudaStream_t stream);
// Build the dynamic-mode records and the active depth ranges from the
// traveltime and weight arrays.
int launch_pack_tables(const KirchDev& K, const float* wsc, const float* wss, const float* wrc,
                       const float* wrs, int4* stab, int4* rtab, uint32_t* srng, uint32_t* rrng,
                       cudaStream_t stream);
// Receivers per group of the fixed-point spread (variant 0) for this
// operator, 0 when the forward does not run that kernel (binned variants,
// single traveltime table, traces too long for shared memory).
int spread_group_size(const KirchDev& K, int L);
// Largest number of contributions any bin of the fixed-point spread can
// receive (valid time and nonzero weight, any model), into *count (device
// word, cleared by the call); 0xffffffff when the forward's spread does not
// run in groups of 8 receivers (L: the padded wavelet length of the forward).
int launch_spread_count(const KirchDev& K, bool dynamic, bool gate, int L, unsigned* count, cudaStream_t stream);
// The forward's prepass alone (mv = m * 2/v or m, and its scale block).
int launch_spread_prepass(const KirchDev& K, bool dynamic, const float* m, cudaStream_t stream);
// Union ranges of groups of 8 receivers from the per-receiver ranges.
int launch_group_ranges(const uint32_t* rrng, uint32_t* grng, int nr, int64_t ncol, cudaStream_t stream);
// The same records with the weights rounded to bf16 (8 bytes each).
int launch_pack_tables_bf16(const KirchDev& K, const float* wsc, const float* wss, const float* wrc,
                            const float* wrs, int2* stab2, int2* rtab2, cudaStream_t stream);
// How many float partial images launch_gather may use, and how many receiver
// splits (partial images) it launches for this geometry.
int64_t gather_partial_elems(const KirchDev& K);
int gather_nsplit(const KirchDev& K, bool dynamic, bool gate);

// Look up and cache, for the current device, the address of the static
// scratch array of kgb_kirchhoff_forward_static (forward_static.cu).
int static_scratch_prepare();

// Device table builder (tables.cu).  Rows are [n][ni] float64.
struct TableGeom {
    int ndim, ny, nx, nz;  // ny = 1 in 2-D
    int64_t ni;
    double hy, hx, hz;     // sample spacings
};
int launch_analytic_rows(const TableGeom& g, const double* yax, const double* xax, const double* zax,
                         const double* pts, int np, double vel, double* trav, double* dist, cudaStream_t s);
// 2-D eikonal traveltime rows of ns sources and nr receivers (pts: grid
// coordinates (ix, iz) of the sources, then of the receivers) into trav_s
// and trav_r, in one launch with the unit-speed table of a point at the
// grid's corner into `corner` (ni values); rhs: ni floats of scratch.
int launch_eikonal_tables(const TableGeom& g, const double* speed, float* rhs, const int* pts, int ns, int nr,
                          double* trav_s, double* trav_r, double* corner, unsigned* err, cudaStream_t s);
// Distance (unit-speed eikonal) rows of the same points from the corner table.
int launch_distance_rows(const TableGeom& g, const double* corner, const int* pts, int ns, int nr, double* dist_s,
                         double* dist_r, cudaStream_t s);
int launch_angle_rows(const TableGeom& g, const double* trav, const double* sign_rows, int np, double* ang,
                      cudaStream_t s);
int launch_fold_rows(int ndim, double maxdist, double amin, double amax, const double* taper21,
                     const double* dist, const double* ang, int64_t n, float* wc, float* ws,
                     unsigned long long* wabs, cudaStream_t s);
int launch_absmax(const double* x, int64_t n, unsigned long long* out, cudaStream_t s);
int launch_finite_check(const double* x, int64_t n, long long* bad, cudaStream_t s);
int launch_quantise(const double* t, int64_t n, double inv_dt, double scale, int32_t* q, int* qmin, cudaStream_t s);
int launch_vscale(const double* vel, int64_t nvel, int64_t ni, float* vs, cudaStream_t s);
int launch_rows_to_reference(const double* rows, int n, int64_t ni, double* out, cudaStream_t s);
int launch_amplitude_rows(const double* dist, int64_t n, double maxdist, int ndim, double* amp, cudaStream_t s);

// Deterministic float64 reductions (solver.cu).
int launch_dot_f64(const float* a, const float* b, int64_t n, double* out, double* block_scratch,
                   cudaStream_t stream);
int dot_scratch_doubles();

}  // namespace kgb

// The operator object behind the opaque C handle.
struct kgb_kirchhoff {
    int ns = 0, nr = 0, nt = 0, nz = 0;
    int64_t ni = 0;
    double dt = 0.0;
    int dynamic = 0;
    int frac_bits = 0;
    int L = 0;                 // padded wavelet length
    float* h_dev = nullptr;    // padded wavelet
    float* hflip_dev = nullptr;// reversed padded wavelet (correlation)
    int32_t* tsq = nullptr;
    int32_t* trq = nullptr;
    float* wsc = nullptr;
    float* wss = nullptr;
    float* wrc = nullptr;
    float* wrs = nullptr;
    float* vscale = nullptr;
    int32_t* izmin = nullptr;
    bool has_gate = false;
    bool nonneg = true;
    float wmax = 1.f;
    int spread_variant = 0;
    float* mv = nullptr;
    unsigned* absmax = nullptr;
    bool trav_ready = false;
    bool dyn_ready = false;
    int4* stab = nullptr;
    int4* rtab = nullptr;
    uint32_t* srng = nullptr;
    uint32_t* rrng = nullptr;
    uint32_t* grng = nullptr;
    int2* stab2 = nullptr;     // bf16-weight records (when bf16_weights), see KirchDev
    int2* rtab2 = nullptr;
    bool bf16_weights = false;
    unsigned long long* wacc = nullptr;  // wide contributions of the split spread, see KirchDev
    bool split_ok = false;
    unsigned* count_buf = nullptr;       // one device word for launch_spread_count
    unsigned max_bin_count = 0;          // its last result
    CUtensorMap stab_map, stab2_map;     // TMA maps over stab / stab2 (see KirchDev::rec_map)
    bool stab_map_ok = false, stab2_map_ok = false;
    int adjoint_variant = 0;             // see KirchDev::adjoint_variant
    // tables built on the device (kgb_kirchhoff_build_tables): [n][ni]
    // float64 rows kept for kgb_kirchhoff_get_table
    double* trav64_s = nullptr;
    double* trav64_r = nullptr;
    double* dist64_s = nullptr;
    double* dist64_r = nullptr;
    double* ang64_s = nullptr;
    double* ang64_r = nullptr;
    double maxdist = 0.0;
    int table_ndim = 0;
    unsigned* err = nullptr;             // device error word of the bounded waits
    int32_t* tq1 = nullptr;    // single traveltime table (trace-major), see KirchDev
    float* tw1 = nullptr;
    float* dcorr = nullptr;    // scratch: correlated data for the adjoint, interleaved pairs (2 x ndata)
    float* partial = nullptr;  // scratch: per-receiver-split partial images
    int64_t partial_elems = 0;
    float* m_stage = nullptr;  // device staging for the host-buffer entry points
    float* d_stage = nullptr;
    cudaStream_t stream = nullptr;  // used by the host-buffer entry points
    // host-buffer entry points: a second compute stream and a copy stream
    // (created on first use) and the events that order the chunks
    static constexpr int kHostChunks = 8;
    cudaStream_t stream2 = nullptr;
    cudaStream_t cstream = nullptr;
    cudaEvent_t ev[kHostChunks + 1] = {};
    int device = 0;

    kgb::KirchDev view() const {
        kgb::KirchDev K;
        K.ns = ns; K.nr = nr; K.nt = nt; K.nz = nz; K.ni = ni; K.frac_bits = frac_bits;
        K.tsq = tsq; K.trq = trq; K.wsc = wsc; K.wss = wss; K.wrc = wrc; K.wrs = wrs;
        K.vscale = vscale; K.izmin = izmin;
        K.nonneg = nonneg ? 1 : 0; K.wmax = wmax; K.mv = mv; K.absmax = absmax;
        K.spread_variant = spread_variant;
        K.stab = stab; K.rtab = rtab; K.srng = srng; K.rrng = rrng; K.grng = grng;
        K.tq1 = tq1; K.tw1 = tw1;
        K.stab2 = bf16_weights ? stab2 : nullptr; K.rtab2 = bf16_weights ? rtab2 : nullptr;
        K.g0 = 0; K.g1 = 1 << 30; K.prepass = 1;
        K.split_ok = split_ok ? 1 : 0; K.wacc = wacc; K.count_out = count_buf;
        K.rec_map = adjoint_variant != 2 ? nullptr
                    : bf16_weights ? (stab2_map_ok ? &stab2_map : nullptr) : (stab_map_ok ? &stab_map : nullptr);
        K.adjoint_variant = adjoint_variant;
        K.err = err;
        return K;
    }
    int64_t npair() const { return (int64_t)ns * nr; }
    int64_t ndata() const { return npair() * nt; }
};
