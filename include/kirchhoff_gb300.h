/*
 * kirchhoff_gb300.h -- C ABI of the GB300-native Kirchhoff demigration /
 * migration operator and of its least-squares solvers.
 *
 * Plain C: opaque handles, raw pointers and sizes, no framework types.
 * Every entry point returns an int status (KGB_OK on success); the message
 * of the last failure on the calling thread is kgb_last_error().
 *
 * Pointers named *_dev are CUDA device pointers (any allocator); pointers
 * named *_host are host memory.  `stream` is a cudaStream_t passed as void*
 * (NULL = the legacy default stream).  Device entry points are asynchronous
 * with respect to the host; *_host entry points synchronise before returning.
 *
 * Reference interfaces (PyLops 2.5.0, paths inside the pylops project):
 *   Kirchhoff.__init__              pylops/waveeqprocessing/kirchhoff.py:234-455
 *   Kirchhoff._matvec / _rmatvec    pylops/waveeqprocessing/kirchhoff.py:1048-1143
 *   _travsrcrec_kirch_(r)matvec     pylops/waveeqprocessing/kirchhoff.py:728-781
 *   _ampsrcrec_kirch_(r)matvec      pylops/waveeqprocessing/kirchhoff.py:784-1001
 *   _KirchhoffCudaHelper            pylops/waveeqprocessing/_kirchhoff_cuda.py:9-489
 *   _Convolve1Dshort                pylops/signalprocessing/convolve1d.py:57-116
 *   CGLS / LSQR                     pylops/optimization/cls_basic.py:334-1351
 */
#ifndef KIRCHHOFF_GB300_H
#define KIRCHHOFF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (mapped to Python exceptions by the host wrapper) ---- */
#define KGB_OK 0
#define KGB_ERR_VALUE 1           /* ValueError: bad sizes, non-finite tables  */
#define KGB_ERR_NOT_IMPLEMENTED 2 /* NotImplementedError                       */
#define KGB_ERR_CUDA 3            /* RuntimeError: a CUDA call failed          */
#define KGB_ERR_MEMORY 4          /* MemoryError: device allocation failed     */
#define KGB_ERR_STATE 5           /* RuntimeError: tables missing, bad handle  */

typedef struct kgb_kirchhoff kgb_kirchhoff; /* opaque operator handle */

/* Library version (major*10000 + minor*100 + patch) and last error text. */
int kgb_version(void);
const char* kgb_last_error(void);

/* Create an operator for ns sources, nr receivers, nt time samples of
 * spacing dt and ni image points whose fastest axis is depth (nz samples):
 * ii = ix*nz + iz in 2-D, (iy*nx + ix)*nz + iz in 3-D.  `wav` is the
 * wavelet as given to the reference constructor and `wavcenter` its centre
 * index; the filter is padded exactly as _Convolve1Dshort does
 * (convolve1d.py:76-88).
 * Replaces: Kirchhoff.__init__ (kirchhoff.py:234-455) for the sizes, the
 * wavelet operator (kirchhoff.py:400-409) and the engine registration
 * (kirchhoff.py:1003-1046). */
int kgb_kirchhoff_create(kgb_kirchhoff** op, int ns, int nr, int nt, int64_t ni, int nz,
                         double dt, int dynamic, const double* wav_host, int nwav,
                         int wavcenter);
int kgb_kirchhoff_destroy(kgb_kirchhoff* op);

/* Upload traveltime tables in the reference layout: trav_srcs (ni, ns) and
 * trav_recs (ni, nr), C order, float64 seconds.  They are stored on the
 * device source-/receiver-major as 32-bit fixed-point sample counts.
 * Replaces: the trav_srcs / trav_recs attributes (kirchhoff.py:310-343) and
 * the per-call to_cupy copies (_kirchhoff_cuda.py:318-328). */
int kgb_kirchhoff_set_traveltimes(kgb_kirchhoff* op, const double* trav_srcs_host,
                                  const double* trav_recs_host);

/* Weight precision of a dynamic operator: bf16 = 1 stores each table entry
 * as an 8-byte record (fixed-point traveltime, cos and sin half-angle
 * weights rounded to bf16) instead of 16 bytes; bf16 = 0 (default) keeps
 * float32 weights.  Traveltimes stay exact.  The bf16 weights change results
 * by about 1e-3 relative (each weight is rounded to 8 significant bits), so
 * float32 is the mode that meets the 1e-5 parity with the reference.
 * Replaces: the float64 amp_* / angle_* tables in the dynamic kernels
 * (kirchhoff.py:784-1001), at half the table bytes. */
int kgb_kirchhoff_set_weight_precision(kgb_kirchhoff* op, int bf16);

/* Single traveltime table: trav (ni, ns*nr) float64 in the reference layout
 * (trav[ii][is*nr + ir], the `trav` array of mode='byot').  Kinematic
 * operators only (a dynamic operator returns KGB_ERR_NOT_IMPLEMENTED, as the
 * reference raises).  The index is the reference's int(t/dt) and the
 * fraction t/dt - int(t/dt) (kept to 2^-19 samples or better); stored
 * trace-major in HBM, 4 bytes per entry (8 if any time is negative).  The
 * operator then spreads and gathers with this table instead of per-source
 * and per-receiver tables.
 * Replaces: itrav/travd (kirchhoff.py:396-398) and _trav_kirch_matvec /
 * _trav_kirch_rmatvec (kirchhoff.py:684-725). */
int kgb_kirchhoff_set_traveltime_table(kgb_kirchhoff* op, const double* trav);

/* Upload the dynamic-mode tables (reference layout, float64): amplitudes and
 * angles (ni, ns) / (ni, nr), velocity (ni), aperture [min, max], angle
 * aperture [min, max] in radians, the 21-sample aperture taper and the
 * per-trace source/receiver x indices six, rix (ns*nr).  Angle tapers,
 * cos/sin of half angles and amplitudes are folded into per-entry weights.
 * Replaces: amp_*, angle_*, vel, aperture, angleaperture, aperturetap, six,
 * rix (kirchhoff.py:287-330, 364-393, 411-439, 448-454). */
int kgb_kirchhoff_set_dynamic(kgb_kirchhoff* op, const double* amp_srcs_host,
                              const double* amp_recs_host, const double* angle_srcs_host,
                              const double* angle_recs_host, const double* vel_host,
                              const double* aperture2_host, const double* angleaperture2_host,
                              const double* aperturetap21_host, const int64_t* six_host,
                              const int64_t* rix_host);

/* Build the tables on the device instead of uploading them: mode 0 =
 * analytic (constant velocity *vel, nvel = 1; 2-D or 3-D), mode 1 = eikonal
 * (2-D or 3-D; vel of ni values in the image order, or one constant), on the
 * operator's grid given by its axes (y of ny samples in 3-D, else NULL; x;
 * z) with sources and receivers (ndim, ns) / (ndim, nr) in the reference's
 * coordinate order ((x, z) or (y, x, z)).  Traveltimes, distances, their
 * gradients, angles and amplitudes are computed as the reference's
 * constructor does and go straight into the operator's fixed-point and
 * folded-weight rows; dynamic operators also take the apertures, the taper
 * and six/rix as in kgb_kirchhoff_set_dynamic.  *maxdist_out receives
 * 1e-2 (max dist_s + max dist_r).  The float64 rows stay on the device for
 * kgb_kirchhoff_get_table.  Eikonal tables solve the fast-marching
 * equations of kgb_eikonal_tables by sweeping (float32 local solves relative
 * to the smallest neighbour); they agree with it to ~1e-7 of the largest
 * time where marching and sweeping pick the same upwind stencils and to
 * ~6e-5 elsewhere.
 * Replaces: Kirchhoff._traveltime_table and the table set-up of
 * Kirchhoff.__init__ (kirchhoff.py:303-393, 503-657); the eikonal solves
 * replace scikit-fmm's travel_time / distance (kirchhoff.py:609-638). */
int kgb_kirchhoff_build_tables(kgb_kirchhoff* op, int mode, int ndim, const double* y_axis, int ny,
                               const double* x_axis, int nx, const double* z_axis, int nz,
                               const double* srcs, const double* recs, const double* vel, int64_t nvel,
                               const double* aperture2_host, const double* angleaperture2_host,
                               const double* aperturetap21_host, const int64_t* six_host,
                               const int64_t* rix_host, double* maxdist_out);

/* One device-built table in the reference layout (ni, n) float64 into
 * out_host: which = 0/1 traveltimes of sources/receivers, 2/3 amplitudes,
 * 4/5 angles (dynamic operators).  KGB_ERR_STATE if the operator's tables
 * were uploaded rather than built.
 * Replaces: reading trav_srcs, trav_recs, amp_srcs, amp_recs, angle_srcs,
 * angle_recs (kirchhoff.py:310-393). */
int kgb_kirchhoff_get_table(kgb_kirchhoff* op, int which, double* out_host);

/* Forward d = K m: spreading along traveltime curves then wavelet
 * convolution.  m_dev (ni) float32, d_dev (ns*nr, nt) float32.
 * Replaces: Kirchhoff._matvec (kirchhoff.py:1048-1094). */
int kgb_kirchhoff_forward(kgb_kirchhoff* op, const float* m_dev, float* d_dev, void* stream);

/* Forward d = K m exactly as kgb_kirchhoff_forward, but the call allocates
 * nothing: its scratch (the model scaled by 2/v and that scale's maximum)
 * lives in a static device array inside the library instead of buffers the
 * operator owns.  For callers that must not call cudaMalloc while they run
 * (a fixed device-memory budget, memory owned by a pool or caching
 * allocator, latency-critical loops).  At most 4,194,304 image points
 * (16 MiB of scratch, held on every GPU where the library's device code is
 * loaded until exit); larger operators get KGB_ERR_VALUE.  All calls on a
 * GPU share the array, so calls that overlap on the GPU race.  The first
 * call on a device looks the array up (make it before any stream capture).
 * No counterpart in the reference. */
int kgb_kirchhoff_forward_static(kgb_kirchhoff* op, const float* m_dev, float* d_dev, void* stream);

/* Adjoint m = K^H d: wavelet correlation then gathering.
 * Replaces: Kirchhoff._rmatvec (kirchhoff.py:1096-1143). */
int kgb_kirchhoff_adjoint(kgb_kirchhoff* op, const float* d_dev, float* m_dev, void* stream);

/* Same as forward/adjoint with host buffers: the copies to and from the
 * device happen inside the call, which returns after the result is on the
 * host.  The copies overlap the kernels (the forward's traces leave in
 * receiver-group chunks as they finish, the adjoint's data arrive in
 * source chunks and are correlated as they land); results equal the
 * device calls bit for bit.  Page-locked host buffers copy at full speed.
 * Replaces: _KirchhoffCudaHelper._matvec_cuda / _rmatvec_cuda
 * (_kirchhoff_cuda.py:443-489) called with numpy arrays. */
int kgb_kirchhoff_forward_host(kgb_kirchhoff* op, const float* m_host, float* d_host);
int kgb_kirchhoff_adjoint_host(kgb_kirchhoff* op, const float* d_host, float* m_host);

/* The two kernels without the wavelet: spreading only (into a zeroed
 * (ns*nr, nt) trace array) and gathering only (from already-correlated data).
 * Replace: the _kirch_matvec / _kirch_rmatvec kernels of
 * kirchhoff.py:728-1001 as registered at kirchhoff.py:1039-1046. */
int kgb_kirchhoff_spread(kgb_kirchhoff* op, const float* m_dev, float* d_dev, void* stream);
int kgb_kirchhoff_gather(kgb_kirchhoff* op, const float* d_dev, float* m_dev, void* stream);

/* Wavelet convolution (adjoint = 0) or correlation (adjoint = 1) of ntr
 * traces of nt samples, 'same' mode with the operator's padded wavelet.
 * Replaces: Kirchhoff.cop._matvec / _rmatvec (convolve1d.py:100-116). */
int kgb_kirchhoff_wavelet(kgb_kirchhoff* op, const float* x_dev, float* y_dev, int adjoint,
                          void* stream);

/* Choose the forward (spreading) kernel: 0 = fixed-point shared-memory
 * accumulation (the default, fastest on every workload measured; it uses
 * the split accumulation of two fire-and-forget atomics per contribution
 * when the operator's bins receive at most 65535 contributions each, see
 * kgb_kirchhoff_info), 1 = warp-binned (one trace per warp), 2 = warp-binned
 * with two traces per warp, 3 = fixed-point with the carry accumulation
 * only (the same traces as 0 bit for bit).  All are deterministic and give
 * the same result up to float32 rounding.  The host-buffer forward overlaps
 * its copies with variants 0 and 3 only.
 * No reference counterpart
 * (the reference has one CUDA kernel per mode, _kirchhoff_cuda.py:55-298);
 * used by the tile autotuner. */
int kgb_kirchhoff_set_variant(kgb_kirchhoff* op, int spread_variant);

/* Adjoint kernel of dynamic operators: 0 (the default) loads each source
 * record in the gather; 1 keeps the next active source's record in flight
 * while the current one's data are read (operators with at most 64 sources);
 * 2 stages the source records through shared memory with TMA bulk-tensor
 * copies.  All three give the same image bit for bit (Kirchhoff.autotune
 * keeps the fastest).  No reference counterpart (the reference's adjoint
 * kernels, _kirchhoff_cuda.py:194-298, read their tables directly). */
int kgb_kirchhoff_set_adjoint_variant(kgb_kirchhoff* op, int variant);

/* Introspection used by the host wrapper and the tests.  info16 receives
 * {ns, nr, nt, ni, fixed-point fraction bits, padded wavelet length,
 *  offset-aperture gate active, dynamic, all times non-negative,
 *  adjoint receiver splits, kernels per forward, kernels per adjoint,
 *  spread variant, split accumulation used by the forward (0/1), most
 *  contributions any forward bin can receive, adjoint variant in use (0-2,
 *  see kgb_kirchhoff_set_adjoint_variant) | error word of the bounded
 *  waits << 2}. */
int kgb_kirchhoff_info(const kgb_kirchhoff* op, int64_t* info16);

/* Deterministic float64 reductions of float32 vectors (fixed launch shape
 * and summation tree, so the result is bit-identical run to run).
 * out_dev receives one double.  Replace: the dot products and norms that
 * CGLS/LSQR take with ncp.linalg.norm / .dot (cls_basic.py:497-564, 976-1136). */
int kgb_dot_f64(const float* a_dev, const float* b_dev, int64_t n, double* out_dev, void* stream);

/* out = base_coef * base + sum_{j<k} coefs[j] * vecs[j] over n floats (base
 * may be NULL; k <= 16; vecs and coefs are host arrays of device pointers
 * and coefficients).  One pass, fixed summation order.  Used by the
 * flexible (network-preconditioned) steps of the learned LSM solve; no
 * reference counterpart. */
int kgb_lincomb_f32(float* out_dev, const float* base_dev, double base_coef, const float* const* vecs,
                    const double* coefs, int k, int64_t n, void* stream);

/* ---- solvers: device-resident CGLS / LSQR ------------------------------
 * The vectors live on the device in float32, every dot product, norm and
 * scalar recurrence is float64 on the device, and one iteration (both
 * operator applications included) is captured in a CUDA graph and replayed
 * without host synchronisation; a device flag retires the remaining
 * replays once the reference's stopping test fires.
 * Replace: CGLS.setup/step/run/finalize (cls_basic.py:432-608) and
 * LSQR.setup/step/run/finalize (cls_basic.py:835-1186). */
typedef struct kgb_solver kgb_solver;

/* kind: 0 = CGLS, 1 = LSQR.  The solver keeps a reference to op. */
int kgb_solver_create(kgb_solver** s, kgb_kirchhoff* op, int kind);
int kgb_solver_destroy(kgb_solver* s);

/* Right preconditioner: with p_dev (ni floats, device, kept by reference;
 * NULL removes it) the solver inverts K diag(p) instead of K, and x, x0 and
 * the model-space state are in the preconditioned variable z (x = p * z),
 * as the reference solvers do on `Kop * Diagonal(p)`
 * (basicoperators/diagonal.py:92-105, linearoperator.py:612-702).  Call
 * before kgb_solver_setup. */
int kgb_solver_set_diagonal(kgb_solver* s, const float* p_dev);

/* Setup with data y (ns*nr*nt) and optional x0 (ni, may be NULL).  params:
 * CGLS {damp, tol}; LSQR {damp, atol, btol, conlim}.  Replaces the setup
 * methods (cls_basic.py:432-506, 835-985). */
int kgb_solver_setup(kgb_solver* s, const float* y_dev, const float* x0_dev,
                     const double* params, int nparams, void* stream);

/* Run up to niter further iterations (replays of the captured iteration,
 * use_graph = 0 launches the same kernels directly).  Replaces run()
 * (cls_basic.py:570-608, 1138-1186). */
int kgb_solver_run(kgb_solver* s, int niter, int use_graph, void* stream);

/* Copy out the current model (ni floats, device) and the scalar state:
 * out16 = {iiter, istop, r1norm, r2norm, anorm, acond, arnorm, xnorm,
 *          var_scalar, kold, 0...}; cost_host receives iiter+1 values of the
 * residual-norm history (may be NULL). */
int kgb_solver_result(kgb_solver* s, float* x_dev, double* out16_host, double* cost_host,
                      int cost_capacity, void* stream);

/* ---- batched least-squares migration ------------------------------------
 * A batch is the block-diagonal operator diag(K_1..K_P) of P kinematic
 * operators (created and filled as above; the batch keeps pointers to their
 * device tables, which must outlive it) over the concatenated models
 * (sum ni_p) and data (sum ns_p*nr_p*nt_p), problem by problem in order.
 * Each application is a single launch per kernel over a work list covering
 * every problem.  kgb_batch_cgls runs CGLS (x0 = 0) on every problem at once
 * with per-problem float64 scalars, replaying one captured iteration in a
 * CUDA-graph WHILE node until every problem meets its stopping rule or has
 * done niter iterations.  cost_host (may be NULL) receives P rows of
 * niter+1 residual norms (row-major), iiter_host / kold_host (may be NULL)
 * P values each.
 * Replaces: a Python loop of LSM problems, each driving CGLS
 * (cls_basic.py:334-708) over its own Kirchhoff operator. */
typedef struct kgb_batch kgb_batch;
int kgb_batch_create(kgb_batch** batch, kgb_kirchhoff* const* ops, int nops);
int kgb_batch_destroy(kgb_batch* batch);
int kgb_batch_sizes(const kgb_batch* batch, int64_t* sizes4); /* {P, model, data, tile} */
int kgb_batch_set_tile(kgb_batch* batch, int receivers_per_item); /* 1, 2, 4 or 8 (autotuner) */
/* Shape of the batched adjoint (autotuner): receiver traveltimes held in
 * registers per image point (4 or 8) and image points per thread (1 or 2).
 * Each point's sum has a fixed order; points per thread leave it unchanged,
 * the receiver count groups it (results agree to float32 rounding).
 * No reference counterpart. */
int kgb_batch_set_gather(kgb_batch* batch, int receivers_in_registers, int points_per_thread);
int kgb_batch_forward(kgb_batch* batch, const float* m_dev, float* d_dev, void* stream);
int kgb_batch_adjoint(kgb_batch* batch, const float* d_dev, float* m_dev, void* stream);
int kgb_batch_cgls(kgb_batch* batch, const float* y_dev, float* x_dev, int niter, double damp, double tol,
                   int use_graph, double* cost_host, int* iiter_host, double* kold_host, void* stream);

/* ---- tensor-core GEMM (U-Net preconditioner) ------------------------------
 * C[m][n] = sum_k A[m][k] B[n][k] (+ bias[n]) (ReLU if flags & 1), A (M x K,
 * leading dimension lda) and B (N x K, ldb) bf16 row-major with K contiguous,
 * C float32 (or bf16 if flags & 2) with leading dimension ldc.  K, lda and
 * ldb must be multiples of 8 and A, B 16-byte aligned.  tcgen05 MMAs with
 * tensor-memory accumulators and TMA-loaded operands; err_dev (may be NULL)
 * is set to 1 if a pipeline wait timed out.  No reference counterpart: the
 * learned preconditioner is new (its training and inference convolutions
 * are lowered to this GEMM). */
int kgb_gemm_bf16_tn(const void* A_dev, const void* B_dev, void* C_dev, int M, int N, int K, int lda, int ldb,
                     int ldc, const float* bias_dev, int flags, int* err_dev, void* stream);

/* Split-K form for reductions over many pixels (weight gradients): C
 * (float32) = A . B^T with the K range cut into `splits` slices (<= 0:
 * chosen to fill the GPU) computed into `work` (splits x M x N floats, at
 * most work_elems; fewer splits if it is smaller) and summed in slice order,
 * so the result is deterministic.  No reference counterpart. */
int kgb_gemm_bf16_tn_splitk(const void* A_dev, const void* B_dev, float* C_dev, int M, int N, int K, int lda,
                            int ldb, int ldc, int splits, float* work_dev, int64_t work_elems, int* err_dev,
                            void* stream);

/* Implicit 3x3 stride-1 convolution (zero padding 1) on the tensor cores:
 * y[p][n] = sum_{tap, c} w[n][tap*Cp + c] x[pixel(p) + sgn*(ky-1, kx-1)][c]
 * (+ bias[n], ReLU if flags & 1, bf16 output if flags & 2, else float32),
 * x NHWC bf16 (B x H x W x C, C % 8 == 0), w bf16 (N x 9*Cp) with Cp = C
 * rounded up to 64 (zero columns), tap = ky*3 + kx, sgn = +1 (flip = 0,
 * forward) or -1 (flip = 1: the transposed convolution that gives a data
 * gradient).  The input is read by 4-D TMA boxes shifted per tap (the
 * padding is the boxes' zero fill): no unfolded copy.  W must divide 128
 * (with H a multiple of 128/W) or be a multiple of 128.  No reference
 * counterpart. */
int kgb_conv3x3_bf16(const void* x_dev, const void* w_dev, void* y_dev, int B, int H, int W, int C, int N, int flip,
                     const float* bias_dev, int flags, int* err_dev, void* stream);

/* Weight gradient of that convolution without an unfolded copy:
 * dW[n][tap*C + c] = sum_p g[p][n] x[pixel(p) + (ky-1, kx-1)][c] (float32,
 * row stride ldw >= 9 C), from gTr (bf16, B H x N x W: the output gradient
 * transposed per image row) and xT3 (bf16, B H x 3 x C x W: the input
 * transposed per image row in three copies, copy kx shifted by kx - 1
 * columns with zero fill), both as kgb_unet_row_transpose writes them.  A
 * tensor-core GEMM whose 128-row A tiles are rows (kx, c) of one image row
 * of xT3 (one TMA box each; the row shift ky is the box's zero fill at the
 * image edges), reduction over pixels (64 per step, one image row segment),
 * split over the pixels into `work` (at least 3 ceil(3 C / 128) 128 x N
 * floats) and summed in slice order (deterministic).  C % 32 == 0,
 * W % 64 == 0.  No reference counterpart. */
/* Data gradient of a 3x3 stride-2 convolution (padding 1) of an input of
 * 2 Hg x 2 Wg pixels: dx (float32, B x 2Hg x 2Wg x N) from the output
 * gradient g (bf16 NHWC, B x Hg x Wg x C, C % 8 == 0) and the transposed
 * weights wt (bf16, N x 9 Cp, as kgb_unet_weights_implicit writes Wti), as
 * four stride-1 implicit convolutions on g, one per output pixel parity
 * (1, 2, 2 and 4 taps), written 2 pixels apart: no unfolded copy.  Wg % 128
 * == 0 (one halo box per kernel row), or Wg = 32 or 64 with Hg a multiple
 * of 128 / Wg (one box of 128 / Wg rows per tap); N <= 128, N % 4 == 0.
 * No reference counterpart. */
int kgb_conv3x3_s2_dgrad_bf16(const void* g_dev, const void* wt_dev, float* dx_dev, int B, int Hg, int Wg, int C,
                              int N, int* err_dev, void* stream);

int kgb_conv3x3_wgrad_bf16(const void* xT3_dev, const void* gTr_dev, float* dW_dev, int B, int H, int W, int C, int N,
                           int ldw, float* work_dev, int64_t work_elems, int* err_dev, void* stream);

/* ---- U-Net helper kernels (NHWC bf16 activations) ------------------------
 * No reference counterpart (the learned preconditioner is new).  A ks x ks
 * convolution (ks 1 or 3, padding ks/2, stride 1 or 2) with weights
 * W[co][(ky*ks+kx)*Cin + ci] runs as GEMMs on unfolded operands:
 *  unfold       out[pd][(ky*ks+kx)*C + c] = src[pixel, c], rows over the
 *               destination grid B x Hd x Wd, columns zero-padded to Kpad;
 *               transposed = 0: source pixel (hd*s+ky-pad, wd*s+kx-pad)
 *               (forward operand); transposed = 1: the source pixel whose
 *               window tap (ky,kx) lands on (hd, wd) (data-gradient operand);
 *  unfold_t     colT[(tap*C + c)][p] over the output pixels p of the
 *               convolution of x (weight-gradient operand);
 *  transpose    out[c][r] = in[r][c] (kind 0 bf16, 1 float32);
 *  weights      bf16 W (Cout x Kpad) and, if Wt != NULL, Wt (Cin x Kg) with
 *               Wt[ci][tap*Cout + co] = W[co][tap*Cin + ci], from float32 W;
 *  weights_implicit  bf16 weights of kgb_conv3x3_bf16 from float32 W
 *               (Cout x Kpad, 3x3): Wi (Cout x 9*Cpi) and, if Wti != NULL,
 *               Wti (Cin x 9*Cpo) for the data gradient, Cpi / Cpo = Cin /
 *               Cout rounded up to 64, zero padded;
 *  relu_grad    g = dy * (y > 0) (relu) or dy, as bf16;
 *  rowsum       out[r] = sum_c in[r][c] (bf16 in, bias gradients; work:
 *               rows x 64 floats of scratch);
 *  upsample     nearest x2 of x into channels [coff, coff+C) of y (Ctot
 *               channels), or (grad) its adjoint from float32 dy;
 *  channels     put (bf16 x into channels of y) or take (float32 channels of
 *               x into y, accumulate optional);
 *  to_bf16      y = x * scale[image] (scale may be NULL);
 *  image_rms    scale[b] = 1/rms of image b (B images of n floats; 0 if zero);
 *  colsum       out[c] = sum_r wt[r] g[r][c] (bf16 g, rows x cols, cols a
 *               multiple of 8 up to 256; wt bf16 or NULL for 1: bias
 *               gradients from the NHWC gradient, or the weight gradient of a
 *               1x1 convolution to one channel; work: 1024 x cols floats;
 *               fixed summation order);
 *  head_forward y[p] = bias[0] + sum_c w[c] x[p][c]: the 1x1 convolution to
 *               one channel (x bf16 NHWC, C % 8 == 0, float32 y);
 *  head_dx      its data gradient dx[p][c] = g[p] w[c] (float32, C % 4 == 0);
 *  conv3x3_c1   3x3 convolution (padding 1) of a one-channel image: y[p][n] =
 *               act(bias[n] + sum_t w[n * kpad + t] x[p + off(t)]), bf16 y,
 *               N % 8 == 0, N <= 128, ReLU if relu;
 *  conv3x3_c1_wgrad  its weight gradient dW[n * kpad + t] = sum_p g[p][n]
 *               x[p + off(t)] (work: 1024 x 9 N floats, fixed order);
 *  row_transpose  per image row r = b H + h of NHWC src (C, W multiples of
 *               8): dst[r][s][c][w] = src[r][w + s - 1][c], s < 3
 *               (shifts = 3, zero outside the row), or dst[r][c][w] =
 *               src[r][w][c] (shifts = 1): the operands of
 *               kgb_conv3x3_wgrad_bf16;
 *  mse          loss = mean (y - t)^2 (double, device), grad = 2 (y - t)/n
 *               (may be NULL), partials: 304 doubles of scratch;
 *  adam         Adam step `step` (1-based) on float32 weights. */
int kgb_unet_unfold(const void* src, void* out, int B, int Hs, int Ws, int C, int Hd, int Wd, int ks, int stride,
                    int transposed, int Kpad, void* stream);
int kgb_unet_unfold_t(const void* x, void* colT, int B, int H, int W, int C, int ks, int stride, void* stream);
int kgb_unet_transpose(const void* in, void* out, int64_t rows, int cols, int64_t ldi, int64_t ldo, int kind,
                       void* stream);
int kgb_unet_weights(const float* W, void* Wb, void* Wt, int Cout, int Cin, int ks, int Kpad, int Kg, void* stream);
int kgb_unet_weights_implicit(const float* W, void* Wi, void* Wti, int Cout, int Cin, int Kpad, void* stream);
int kgb_unet_relu_grad(const float* dy, const void* y, void* g, int64_t n, int relu, void* stream);
int kgb_unet_rowsum(const void* in, float* out, int rows, int64_t cols, float* work, void* stream);
int kgb_unet_upsample(const void* x, void* y, int B, int H, int W, int C, int Ctot, int coff, int grad,
                      void* stream);
int kgb_unet_channels(const void* x, void* y, int64_t P, int C, int Ctot, int coff, int take, int accumulate,
                      void* stream);
int kgb_unet_to_bf16(const float* x, void* y, int64_t n, int B, const float* scale, void* stream);
int kgb_unet_image_rms(const float* x, int64_t n, int B, float* scale, void* stream);
int kgb_unet_row_transpose(const void* src, void* dst, int B, int H, int W, int C, int shifts, void* stream);
int kgb_unet_colsum(const void* g, const void* wt, float* out, int64_t rows, int cols, float* work, void* stream);
int kgb_unet_head_forward(const void* x, const void* w, const float* bias, float* y, int64_t P, int C, void* stream);
int kgb_unet_head_dx(const void* g, const void* w, float* dx, int64_t P, int C, void* stream);
int kgb_unet_conv3x3_c1(const void* x, const void* w, const void* bias, void* y, int B, int H, int W, int N, int kpad,
                        int relu, void* stream);
int kgb_unet_conv3x3_c1_wgrad(const void* x, const void* g, float* dW, int B, int H, int W, int N, int kpad,
                              float* work, void* stream);
int kgb_unet_mse(const float* y, const float* t, float* grad, int64_t n, double* partials, double* loss,
                 void* stream);
int kgb_unet_adam(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                  int step, void* stream);

/* ---- 2-D non-stationary convolution (image-domain Hessian with PSFs) ----
 * x, y: (nx, nz) float32 device arrays (z fastest); hs: (nhx, nhz, hx, hz)
 * float32 device filters on the coarse grid (ohx + k dhx, ohz + l dhz),
 * hx and hz odd.  adjoint = 0: forward (the filter of each input point
 * spread around it), 1: adjoint.  Bilinear interpolation of the four
 * neighbouring filters, edge filters with weights 1/2 outside the coarse
 * grid.  Both directions are gathers (deterministic, no atomics); y is
 * overwritten.
 * Replaces: NonStationaryConvolve2D._matvec_rmatvec and its numba-CUDA
 * kernel (signalprocessing/nonstatconvolve2d.py:177-300,
 * _nonstatconvolve2d_cuda.py:6-111). */
int kgb_nsconv2d_apply(const float* x_dev, float* y_dev, const float* hs_dev, int nx, int nz, int nhx, int nhz,
                       int hx, int hz, double ohx, double ohz, double dhx, double dhz, int adjoint, void* stream);

/* ---- table builder ------------------------------------------------------
 * First-arrival traveltimes (and, if dist_out != NULL, distances) from npts
 * point sources by fast marching on a regular grid of ndim (2 or 3) axes
 * `dims` (C order, depth fastest) with spacings `dsamp` and velocity
 * `speed` (prod(dims) values).  pts holds npts x ndim grid indices.  Output
 * tables are (prod(dims), npts) in C order, i.e. the reference's
 * trav_srcs / dist_srcs layout.  One OpenMP thread per point source
 * (nthreads <= 0: all host threads).
 * Replaces: the skfmm.travel_time / skfmm.distance loop of
 * Kirchhoff._traveltime_table (kirchhoff.py:609-638). */
int kgb_eikonal_tables(int ndim, const int* dims, const double* dsamp, const double* speed, int npts,
                       const int* pts, double* trav_out, double* dist_out, int order, int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* KIRCHHOFF_GB300_H */
