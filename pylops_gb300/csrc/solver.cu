// Device-resident CGLS and LSQR (pylops/optimization/cls_basic.py:334-1351).
//
// Vectors are float32 on the device; every dot product, norm and scalar
// recurrence is float64 and stays on the device, so an iteration needs no
// host synchronisation.  One iteration (two operator applications plus the
// vector and scalar kernels) is captured once into the body of a CUDA-graph
// WHILE node; a scalar kernel at the end of the body evaluates the
// reference's stopping test and sets the node's condition, so a whole solve
// is a single graph launch.
//
// Reductions are deterministic: fixed grid, per-block float64 partials and a
// fixed-order final sum.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>
#include <vector>

#include "dfacc.cuh"
#include "kgb_internal.h"

namespace kgb {
namespace sk {

constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 304;  // 2 x 152 SMs; fixed => deterministic sums

struct SolverState {
    // shared
    int iiter, istop, niter_setup, target, active, kind;
    double damp, dampsq;
    // LSQR
    double alfa, beta, inv_alfa, inv_beta, rhobar, phibar, bnorm, rnorm, r1norm, r2norm;
    double anorm, acond, arnorm, arnorm0, ddnorm, res2, xnorm, xxnorm, z, cs2, sn2;
    double atol, btol, ctol, var_scalar, t1, t2, rho, psi, tau, phi, theta;
    double test1, test2, test3;
    int beta_pos, alfa_pos;
    // CGLS
    double kold, k, a, b, tol, damp_setup;
    double sums[4];
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum in a fixed order; result valid in thread 0.
__device__ double block_sum(double v) {
    __shared__ double sh[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    v = warp_sum(v);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    const int nw = blockDim.x >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (warp == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

__global__ void __launch_bounds__(kRedThreads)
dot_partial_kernel(const float* __restrict__ a, const float* __restrict__ b, int64_t n,
                   double* __restrict__ partials) {
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dacc.add_prod(a[i], b[i]);
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// Fixed-order sum of `np` partials into *out (one block).
__device__ double sum_partials(const double* __restrict__ partials, int np) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc += partials[i];
    return block_sum(acc);
}

__global__ void __launch_bounds__(kRedThreads)
dot_final_kernel(const double* __restrict__ partials, int np, double* __restrict__ out) {
    const double s = sum_partials(partials, np);
    if (threadIdx.x == 0) *out = s;
}

// ----------------------------------------------------------------- LSQR
// u = ub - alfa*u, sum u^2 (cls_basic.py:1009-1015)
__global__ void __launch_bounds__(kRedThreads)
lsqr_u_kernel(float* __restrict__ u, const float* __restrict__ ub, int64_t n,
              const SolverState* __restrict__ st, double* __restrict__ partials) {
    if (!st->active) return;
    const float alfa = (float)st->alfa;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float v = ub[i] - alfa * u[i];
        u[i] = v;
        dacc.add_prod(v, v);
    }
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// beta = ||u||; anorm update (cls_basic.py:1016-1024)
__global__ void __launch_bounds__(kRedThreads)
lsqr_beta_kernel(SolverState* st, const double* __restrict__ partials, int np) {
    if (!st->active) return;
    const double s = sum_partials(partials, np);
    if (threadIdx.x != 0) return;
    const double beta = sqrt(s);
    st->beta = beta;
    st->beta_pos = beta > 0.0;
    if (beta > 0.0) {
        st->inv_beta = 1.0 / beta;
        st->anorm = sqrt(st->anorm * st->anorm + st->alfa * st->alfa + beta * beta + st->damp * st->damp);
    }
}

__global__ void scale_kernel(float* __restrict__ x, int64_t n, const SolverState* __restrict__ st, int which) {
    if (!st->active) return;
    float f;
    if (which == 0) {
        if (!st->beta_pos) return;
        f = (float)st->inv_beta;
    } else {
        if (!(st->beta_pos && st->alfa_pos)) return;
        f = (float)st->inv_alfa;
    }
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= f;
}

// v = vb - beta*v, sum v^2 (cls_basic.py:1025-1034)
__global__ void __launch_bounds__(kRedThreads)
lsqr_v_kernel(float* __restrict__ v, const float* __restrict__ vb, int64_t n,
              const SolverState* __restrict__ st, double* __restrict__ partials) {
    if (!st->active || !st->beta_pos) return;
    const float beta = (float)st->beta;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float t = vb[i] - beta * v[i];
        v[i] = t;
        dacc.add_prod(t, t);
    }
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// alfa = ||v|| and the two plane rotations (cls_basic.py:1035-1062)
__global__ void __launch_bounds__(kRedThreads)
lsqr_rot_kernel(SolverState* st, const double* __restrict__ partials, int np) {
    if (!st->active) return;
    const double s = st->beta_pos ? sum_partials(partials, np) : 0.0;
    if (threadIdx.x != 0) return;
    if (st->beta_pos) {
        st->alfa = sqrt(s);
        st->alfa_pos = st->alfa > 0.0;
        if (st->alfa_pos) st->inv_alfa = 1.0 / st->alfa;
    } else {
        st->alfa_pos = 0;
    }
    const double damp = st->damp;
    const double rhobar1 = sqrt(st->rhobar * st->rhobar + damp * damp);
    const double cs1 = st->rhobar / rhobar1;
    const double sn1 = damp / rhobar1;
    st->psi = sn1 * st->phibar;
    st->phibar = cs1 * st->phibar;
    const double rho = sqrt(rhobar1 * rhobar1 + st->beta * st->beta);
    const double cs = rhobar1 / rho;
    const double sn = st->beta / rho;
    st->theta = sn * st->alfa;
    st->rhobar = -cs * st->alfa;
    st->phi = cs * st->phibar;
    st->phibar = sn * st->phibar;
    st->tau = sn * st->phi;
    st->rho = rho;
    st->t1 = st->phi / rho;
    st->t2 = -st->theta / rho;
}

// v /= alfa; sum w_old^2; x += t1*w; w = v + t2*w (cls_basic.py:1064-1081)
__global__ void __launch_bounds__(kRedThreads)
lsqr_xw_kernel(float* __restrict__ x, float* __restrict__ w, float* __restrict__ v, int64_t n,
               const SolverState* __restrict__ st, double* __restrict__ partials) {
    if (!st->active) return;
    const bool scale_v = st->beta_pos && st->alfa_pos;
    const float inv_alfa = (float)st->inv_alfa;
    const float t1 = (float)st->t1, t2 = (float)st->t2;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float vi = v[i];
        if (scale_v) {
            vi *= inv_alfa;
            v[i] = vi;
        }
        const float wi = w[i];
        dacc.add_prod(wi, wi);
        x[i] = x[i] + t1 * wi;
        w[i] = vi + t2 * wi;
    }
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

__device__ void lsqr_tail(SolverState* st, double dk2, double* cost) {
    st->ddnorm = st->ddnorm + dk2;
    st->var_scalar = st->var_scalar + dk2;
    const double delta = st->sn2 * st->rho;
    const double gambar = -st->cs2 * st->rho;
    const double rhs = st->phi - delta * st->z;
    const double zbar = rhs / gambar;
    st->xnorm = sqrt(st->xxnorm + zbar * zbar);
    const double gamma = sqrt(gambar * gambar + st->theta * st->theta);
    st->cs2 = gambar / gamma;
    st->sn2 = st->theta / gamma;
    st->z = rhs / gamma;
    st->xxnorm = st->xxnorm + st->z * st->z;
    st->acond = st->anorm * sqrt(st->ddnorm);
    const double res1 = st->phibar * st->phibar;
    st->res2 = st->res2 + st->psi * st->psi;
    st->rnorm = sqrt(res1 + st->res2);
    st->arnorm = st->alfa * fabs(st->tau);
    const double r1sq = st->rnorm * st->rnorm - st->dampsq * st->xxnorm;
    double r1norm = sqrt(fabs(r1sq));
    cost[st->iiter + 1] = r1norm;
    if (r1sq < 0) r1norm = -r1norm;
    st->r1norm = r1norm;
    st->r2norm = st->rnorm;
    st->test1 = st->rnorm / st->bnorm;
    st->test2 = st->arnorm / st->arnorm0;
    st->test3 = 1.0 / st->acond;
    const double t1 = st->test1 / (1.0 + st->anorm * st->xnorm / st->bnorm);
    const double rtol = st->btol + st->atol * st->anorm * st->xnorm / st->bnorm;
    int istop = st->istop;
    if (st->iiter >= st->niter_setup) istop = 7;
    if (1.0 + st->test3 <= 1.0) istop = 6;
    if (1.0 + st->test2 <= 1.0) istop = 5;
    if (1.0 + t1 <= 1.0) istop = 4;
    if (st->test3 <= st->ctol) istop = 3;
    if (st->test2 <= st->atol) istop = 2;
    if (st->test1 <= rtol) istop = 1;
    st->istop = istop;
    st->iiter += 1;
}

__global__ void __launch_bounds__(kRedThreads)
lsqr_tail_kernel(SolverState* st, const double* __restrict__ partials, int np, double* cost,
                 cudaGraphConditionalHandle handle, int use_handle) {
    if (st->active) {
        const double s = sum_partials(partials, np);
        if (threadIdx.x == 0) {
            const double dk2 = s / (st->rho * st->rho);
            lsqr_tail(st, dk2, cost);
            st->active = (st->istop == 0 && st->iiter < st->target) ? 1 : 0;
        }
    }
    if (threadIdx.x == 0 && use_handle) cudaGraphSetConditional(handle, st->active ? 1u : 0u);
}

// ----------------------------------------------------------------- CGLS
__global__ void __launch_bounds__(kRedThreads)
sq_partial_kernel(const float* __restrict__ a, int64_t n, const SolverState* __restrict__ st,
                  double* __restrict__ partials) {
    if (!st->active) return;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dacc.add_prod(a[i], a[i]);
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// x += a c, sum x^2 (cls_basic.py:529, 558-563)
__global__ void __launch_bounds__(kRedThreads)
cgls_x_kernel(float* __restrict__ x, const float* __restrict__ c, int64_t n,
              const SolverState* __restrict__ st, double* __restrict__ partials) {
    if (!st->active) return;
    const float a = (float)st->a;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float t = x[i] + a * c[i];
        x[i] = t;
        dacc.add_prod(t, t);
    }
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// s -= a q, sum s^2 (cls_basic.py:530)
__global__ void __launch_bounds__(kRedThreads)
cgls_s_kernel(float* __restrict__ s, const float* __restrict__ q, int64_t n,
              const SolverState* __restrict__ st, double* __restrict__ partials) {
    if (!st->active) return;
    const float a = (float)st->a;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float t = s[i] - a * q[i];
        s[i] = t;
        dacc.add_prod(t, t);
    }
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// r = K^H s - damp x, sum r^2 (cls_basic.py:531, 542-544)
__global__ void __launch_bounds__(kRedThreads)
cgls_r_kernel(float* __restrict__ r, const float* __restrict__ x, int64_t n,
              const SolverState* __restrict__ st, double* __restrict__ partials) {
    if (!st->active) return;
    const float damp = (float)st->dampsq;
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float t = r[i] - damp * x[i];
        r[i] = t;
        dacc.add_prod(t, t);
    }
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

// c = r + b c (cls_basic.py:546-550)
__global__ void cgls_c_kernel(float* __restrict__ c, const float* __restrict__ r, int64_t n,
                              const SolverState* __restrict__ st) {
    if (!st->active) return;
    const float b = (float)st->b;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        c[i] = r[i] + b * c[i];
}

__global__ void cgls_tail_kernel(SolverState* st, cudaGraphConditionalHandle handle, int use_handle) {
    if (st->active) {
        st->kold = st->k;
        st->iiter += 1;
        st->active = (st->iiter < st->target && st->kold > st->tol) ? 1 : 0;
    }
    if (use_handle) cudaGraphSetConditional(handle, st->active ? 1u : 0u);
}

__global__ void set_target_kernel(SolverState* st, int add, cudaGraphConditionalHandle handle, int use_handle) {
    st->target = st->iiter + add;
    if (st->kind == 0)
        st->active = (st->iiter < st->target && st->kold > st->tol) ? 1 : 0;
    else
        st->active = (st->iiter < st->target && st->istop == 0) ? 1 : 0;
    if (use_handle) cudaGraphSetConditional(handle, st->active ? 1u : 0u);
}

int grid_for(int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>(kRedBlocks, (n + kRedThreads - 1) / kRedThreads)); }

}  // namespace sk

using namespace sk;

int dot_scratch_doubles() { return kRedBlocks; }

int launch_dot_f64(const float* a, const float* b, int64_t n, double* out, double* partials, cudaStream_t s) {
    const int g = grid_for(n);
    dot_partial_kernel<<<g, kRedThreads, 0, s>>>(a, b, n, partials);
    dot_final_kernel<<<1, kRedThreads, 0, s>>>(partials, g, out);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

}  // namespace kgb

using namespace kgb;

struct kgb_solver {
    kgb_kirchhoff* op = nullptr;
    int kind = 0;  // 0 CGLS, 1 LSQR
    int64_t n = 0, m = 0;  // model and data sizes
    // model space
    float *x = nullptr, *mv1 = nullptr, *mv2 = nullptr, *mv3 = nullptr;
    // data space
    float *dv1 = nullptr, *dv2 = nullptr;
    SolverState* st = nullptr;
    double* partials = nullptr;  // 4 * kRedBlocks
    double* cost = nullptr;
    double* cost1 = nullptr;
    int cost_cap = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle handle = 0;
    bool setup_done = false;
    // optional right preconditioner: the solver then works on K diag(pdiag)
    const float* pdiag = nullptr;
    float* mvp = nullptr;  // model-space scratch for pdiag * v
};

namespace kgb {
namespace sk {

int ensure_cost(kgb_solver* s, int need) {
    if (need <= s->cost_cap) return KGB_OK;
    int cap = std::max(need, 2 * s->cost_cap + 64);
    double *c = nullptr, *c1 = nullptr;
    KGB_CUDA_TRY(cudaMalloc(&c, cap * sizeof(double)));
    KGB_CUDA_TRY(cudaMalloc(&c1, cap * sizeof(double)));
    KGB_CUDA_TRY(cudaMemset(c, 0, cap * sizeof(double)));
    KGB_CUDA_TRY(cudaMemset(c1, 0, cap * sizeof(double)));
    if (s->cost) {
        KGB_CUDA_TRY(cudaMemcpy(c, s->cost, s->cost_cap * sizeof(double), cudaMemcpyDeviceToDevice));
        KGB_CUDA_TRY(cudaMemcpy(c1, s->cost1, s->cost_cap * sizeof(double), cudaMemcpyDeviceToDevice));
        cudaFree(s->cost);
        cudaFree(s->cost1);
    }
    s->cost = c;
    s->cost1 = c1;
    s->cost_cap = cap;
    // the captured graph bakes the cost pointers in
    if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
    if (s->graph) { cudaGraphDestroy(s->graph); s->graph = nullptr; }
    return KGB_OK;
}

// out = p (.) v; out may be v (in-place scaling), so neither is restrict
__global__ void diag_mul_kernel(float* out, const float* __restrict__ p, const float* v, int64_t n) {
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = p[i] * v[i];
}

// The operator the solver inverts: K, or K diag(p) with a right preconditioner.
int op_forward(kgb_solver* s, const float* v, float* out, cudaStream_t stream) {
    if (!s->pdiag) return kgb_kirchhoff_forward(s->op, v, out, stream);
    diag_mul_kernel<<<grid_for(s->n), kRedThreads, 0, stream>>>(s->mvp, s->pdiag, v, s->n);
    KGB_CUDA_TRY(cudaGetLastError());
    return kgb_kirchhoff_forward(s->op, s->mvp, out, stream);
}

int op_adjoint(kgb_solver* s, const float* u, float* out, cudaStream_t stream) {
    int rc = kgb_kirchhoff_adjoint(s->op, u, out, stream);
    if (rc || !s->pdiag) return rc;
    diag_mul_kernel<<<grid_for(s->n), kRedThreads, 0, stream>>>(out, s->pdiag, out, s->n);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

// One LSQR iteration's launches on `stream` (captured or direct).
int enqueue_iteration(kgb_solver* s, cudaStream_t stream, int use_handle) {
    const int gn = grid_for(s->n), gm = grid_for(s->m);
    double* P0 = s->partials;
    double* P1 = s->partials + kRedBlocks;
    int rc;
    {  // LSQR: x, v=mv1, w=mv2, vb=mv3; u=dv1, ub=dv2
        if ((rc = op_forward(s, s->mv1, s->dv2, stream))) return rc;
        lsqr_u_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, s->dv2, s->m, s->st, P0);
        lsqr_beta_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P0, gm);
        scale_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, s->m, s->st, 0);
        if ((rc = op_adjoint(s, s->dv1, s->mv3, stream))) return rc;
        lsqr_v_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->mv3, s->n, s->st, P0);
        lsqr_rot_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P0, gn);
        lsqr_xw_kernel<<<gn, kRedThreads, 0, stream>>>(s->x, s->mv2, s->mv1, s->n, s->st, P1);
        lsqr_tail_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P1, gn, s->cost, s->handle, use_handle);
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

// The CGLS body is written separately because its reductions mix sizes.

__global__ void __launch_bounds__(kRedThreads)
cgls_a2_kernel(SolverState* st, const double* __restrict__ pq, int npq, const double* __restrict__ pc, int npc) {
    if (!st->active) return;
    const double qq = sum_partials(pq, npq);
    const double cc = sum_partials(pc, npc);
    if (threadIdx.x == 0) st->a = st->kold / (qq + st->dampsq * cc);
}

__global__ void __launch_bounds__(kRedThreads)
cgls_b2_kernel(SolverState* st, const double* __restrict__ pr, int npr, const double* __restrict__ ps,
               int nps, const double* __restrict__ px, int npx, double* cost, double* cost1) {
    if (!st->active) return;
    const double k = sum_partials(pr, npr);
    const double ss = sum_partials(ps, nps);
    const double xx = sum_partials(px, npx);
    if (threadIdx.x == 0) {
        st->k = k;
        st->b = k / st->kold;
        const double c0 = sqrt(ss);
        cost[st->iiter + 1] = c0;
        cost1[st->iiter + 1] = sqrt(c0 * c0 + st->dampsq * fabs(xx));
    }
}

int enqueue_cgls_iteration(kgb_solver* s, cudaStream_t stream, int use_handle) {
    const int gn = grid_for(s->n), gm = grid_for(s->m);
    double* P0 = s->partials;
    double* P1 = s->partials + kRedBlocks;
    double* P2 = s->partials + 2 * kRedBlocks;
    double* P3 = s->partials + 3 * kRedBlocks;
    int rc;
    // x, c=mv1, r=mv2; s=dv1, q=dv2
    sq_partial_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv2, s->m, s->st, P0);
    sq_partial_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->n, s->st, P1);
    cgls_a2_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P0, gm, P1, gn);
    cgls_x_kernel<<<gn, kRedThreads, 0, stream>>>(s->x, s->mv1, s->n, s->st, P2);
    cgls_s_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, s->dv2, s->m, s->st, P3);
    if ((rc = op_adjoint(s, s->dv1, s->mv2, stream))) return rc;
    cgls_r_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv2, s->x, s->n, s->st, P0);
    cgls_b2_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P0, gn, P3, gm, P2, gn, s->cost, s->cost1);
    cgls_c_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->mv2, s->n, s->st);
    if ((rc = op_forward(s, s->mv1, s->dv2, stream))) return rc;
    cgls_tail_kernel<<<1, 1, 0, stream>>>(s->st, s->handle, use_handle);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int enqueue(kgb_solver* s, cudaStream_t stream, int use_handle) {
    return s->kind == 1 ? enqueue_iteration(s, stream, use_handle) : enqueue_cgls_iteration(s, stream, use_handle);
}

__global__ void cond_from_state_kernel(const SolverState* st, cudaGraphConditionalHandle handle) {
    cudaGraphSetConditional(handle, st->active ? 1u : 0u);
}

// Graph: [condition <- state.active] -> WHILE(condition) { iteration }.
// The WHILE node's condition is reset to its default (0) at every launch, so
// the first node of the graph sets it from the device state that
// set_target_kernel prepared.
int build_graph(kgb_solver* s, cudaStream_t stream) {
    if (s->exec) return KGB_OK;
    cudaGraph_t g = nullptr;
    KGB_CUDA_TRY(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "cudaGraphConditionalHandleCreate"); }
    s->handle = h;
    e = cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "cudaStreamBeginCaptureToGraph(init)"); }
    cond_from_state_kernel<<<1, 1, 0, stream>>>(s->st, h);
    cudaError_t le = cudaGetLastError();
    cudaGraph_t tmp = nullptr;
    e = cudaStreamEndCapture(stream, &tmp);
    if (le != cudaSuccess || e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(le != cudaSuccess ? le : e, "capture init node"); }
    cudaGraphNode_t init = nullptr;
    size_t nn = 1;
    e = cudaGraphGetNodes(g, &init, &nn);
    if (e != cudaSuccess || nn != 1) { cudaGraphDestroy(g); return set_error(KGB_ERR_CUDA, "graph init node lookup failed"); }
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t wnode;
    e = cudaGraphAddNode(&wnode, g, &init, nullptr, 1, &cp);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "cudaGraphAddNode(while)"); }
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "cudaStreamBeginCaptureToGraph"); }
    int rc = enqueue(s, stream, 1);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(stream, &captured);
    if (rc != KGB_OK) { cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) { cudaGraphDestroy(g); return cuda_error(e, "cudaStreamEndCapture"); }
    e = cudaGraphInstantiate(&s->exec, g, 0);
    if (e != cudaSuccess) { cudaGraphDestroy(g); s->exec = nullptr; return cuda_error(e, "cudaGraphInstantiate"); }
    s->graph = g;
    return KGB_OK;
}

__global__ void init_state_kernel(SolverState* st, int kind, int niter_setup, double p0, double p1, double p2, double p3) {
    SolverState z = {};
    z.kind = kind;
    z.niter_setup = niter_setup;
    if (kind == 1) {
        z.damp = p0; z.dampsq = p0 * p0; z.atol = p1; z.btol = p2;
        z.ctol = p3 > 0 ? 1.0 / p3 : 0.0;
        z.cs2 = -1.0; z.sn2 = 0.0;
    } else {
        z.damp_setup = p0; z.damp = p0; z.dampsq = p0 * p0; z.tol = p1;
    }
    *st = z;
}

// LSQR setup tail: beta from P0 (||u||^2), scale later; see cls_basic.py:944-985
__global__ void __launch_bounds__(kRedThreads)
lsqr_setup_beta_kernel(SolverState* st, const double* __restrict__ p, int np) {
    const double s = sum_partials(p, np);
    if (threadIdx.x == 0) {
        st->alfa = 0.0;
        st->beta = sqrt(s);
        st->beta_pos = st->beta > 0.0;
        if (st->beta_pos) st->inv_beta = 1.0 / st->beta;
        st->active = 1;
    }
}

__global__ void __launch_bounds__(kRedThreads)
lsqr_setup_alfa_kernel(SolverState* st, const double* __restrict__ p, int np, double* cost) {
    const double s = st->beta_pos ? sum_partials(p, np) : 0.0;
    if (threadIdx.x == 0) {
        if (st->beta_pos) {
            st->alfa = sqrt(s);
            st->alfa_pos = st->alfa > 0.0;
            if (st->alfa_pos) st->inv_alfa = 1.0 / st->alfa;
        } else {
            st->alfa = 0.0;
            st->alfa_pos = 0;
        }
        st->arnorm = st->alfa * st->beta;
        st->arnorm0 = st->arnorm;
        st->rhobar = st->alfa;
        st->phibar = st->beta;
        st->bnorm = st->beta;
        st->rnorm = st->beta;
        st->r1norm = st->beta;
        st->r2norm = st->beta;
        cost[0] = st->rnorm;
        st->iiter = 0;
        st->istop = 0;
        st->active = 0;
    }
}

__global__ void scale_by_kernel(float* __restrict__ x, int64_t n, const SolverState* __restrict__ st, int which) {
    float f;
    if (which == 0) { if (!st->beta_pos) return; f = (float)st->inv_beta; }
    else { if (!(st->beta_pos && st->alfa_pos)) return; f = (float)st->inv_alfa; }
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= f;
}

__global__ void copy_if_beta_zero_kernel(float* __restrict__ v, const float* __restrict__ x, int64_t n,
                                         const SolverState* __restrict__ st) {
    if (st->beta_pos) return;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        v[i] = x[i];
}

__global__ void sub_kernel(float* __restrict__ out, const float* __restrict__ a, const float* __restrict__ b, int64_t n) {
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}

__global__ void axpy_kernel(float* __restrict__ y, const float* __restrict__ x, float a, int64_t n) {
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] += a * x[i];
}

__global__ void __launch_bounds__(kRedThreads)
cgls_setup_kernel(SolverState* st, const double* __restrict__ pcc, int npc, const double* __restrict__ pss,
                  int nps, const double* __restrict__ pxx, int npx, double* cost, double* cost1) {
    const double cc = sum_partials(pcc, npc);
    const double ss = sum_partials(pss, nps);
    const double xx = pxx ? sum_partials(pxx, npx) : 0.0;
    if (threadIdx.x == 0) {
        st->kold = fabs(cc);
        cost[0] = sqrt(ss);
        cost1[0] = sqrt(ss + st->damp_setup * fabs(xx));  // cls_basic.py:498-503 (unsquared damp)
        st->iiter = 0;
        st->active = 0;
    }
}

__global__ void __launch_bounds__(kRedThreads)
sq_partial_plain_kernel(const float* __restrict__ a, int64_t n, double* __restrict__ partials) {
    DFAcc dacc;
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dacc.add_prod(a[i], a[i]);
    double acc = block_sum(dacc.value());
    if (threadIdx.x == 0) partials[blockIdx.x] = acc;
}

}  // namespace sk
}  // namespace kgb

using namespace kgb::sk;

namespace kgb {
namespace sk {

constexpr int kMaxComb = 16;
struct CombArgs {
    const float* v[kMaxComb];
    float c[kMaxComb];
};

// out = c0 * base + sum_j c[j] v[j] (base may be NULL), summed in index order
__global__ void lincomb_kernel(float* __restrict__ out, const float* __restrict__ base, float c0, CombArgs a, int k,
                               int64_t n) {
    #pragma unroll 4
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        float acc = base ? c0 * base[i] : 0.f;
        for (int j = 0; j < k; ++j) acc = fmaf(a.c[j], a.v[j][i], acc);
        out[i] = acc;
    }
}

}  // namespace sk
}  // namespace kgb

extern "C" {

int kgb_lincomb_f32(float* out, const float* base, double base_coef, const float* const* vecs, const double* coefs,
                    int k, int64_t n, void* stream) {
    if (!out || k < 0 || k > sk::kMaxComb || n <= 0 || (k > 0 && (!vecs || !coefs)))
        return set_error(KGB_ERR_VALUE, "lincomb: bad arguments (k <= 16)");
    sk::CombArgs a;
    for (int j = 0; j < sk::kMaxComb; ++j) {
        a.v[j] = j < k ? vecs[j] : nullptr;
        a.c[j] = j < k ? (float)coefs[j] : 0.f;
        if (j < k && !vecs[j]) return set_error(KGB_ERR_VALUE, "lincomb: null vector");
    }
    sk::lincomb_kernel<<<grid_for(n), kRedThreads, 0, (cudaStream_t)stream>>>(out, base, (float)base_coef, a, k, n);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

int kgb_dot_f64(const float* a, const float* b, int64_t n, double* out, void* stream) {
    if (!a || !b || !out) return set_error(KGB_ERR_VALUE, "dot: null pointer");
    static thread_local double* scratch = nullptr;
    static thread_local int scratch_dev = -1;
    int dev = 0;
    KGB_CUDA_TRY(cudaGetDevice(&dev));
    if (!scratch || scratch_dev != dev) {
        KGB_CUDA_TRY(cudaMalloc(&scratch, kRedBlocks * sizeof(double)));
        scratch_dev = dev;
    }
    return launch_dot_f64(a, b, n, out, scratch, (cudaStream_t)stream);
}

int kgb_solver_create(kgb_solver** out, kgb_kirchhoff* op, int kind) {
    if (!out || !op) return set_error(KGB_ERR_VALUE, "solver_create: null pointer");
    if (kind != 0 && kind != 1) return set_error(KGB_ERR_VALUE, "solver_create: kind must be 0 (CGLS) or 1 (LSQR)");
    *out = nullptr;
    kgb_solver* s = new kgb_solver();
    s->op = op;
    s->kind = kind;
    s->n = op->ni;
    s->m = op->ndata();
    cudaError_t e = cudaSuccess;
    auto A = [&](float** p, int64_t n) { if (e == cudaSuccess) e = cudaMalloc(p, (size_t)n * sizeof(float)); };
    A(&s->x, s->n); A(&s->mv1, s->n); A(&s->mv2, s->n); A(&s->mv3, s->n);
    A(&s->dv1, s->m); A(&s->dv2, s->m);
    if (e == cudaSuccess) e = cudaMalloc(&s->st, sizeof(SolverState));
    if (e == cudaSuccess) e = cudaMalloc(&s->partials, 4 * kRedBlocks * sizeof(double));
    if (e != cudaSuccess) {
        int rc = cuda_error(e, "solver_create: allocation");
        kgb_solver_destroy(s);
        return rc;
    }
    int rc = ensure_cost(s, 64);
    if (rc) { kgb_solver_destroy(s); return rc; }
    *out = s;
    return KGB_OK;
}

int kgb_solver_destroy(kgb_solver* s) {
    if (!s) return KGB_OK;
    if (s->exec) cudaGraphExecDestroy(s->exec);
    if (s->graph) cudaGraphDestroy(s->graph);
    void* ptrs[] = {s->x, s->mv1, s->mv2, s->mv3, s->dv1, s->dv2, s->st, s->partials, s->cost, s->cost1, s->mvp};
    for (void* p : ptrs) if (p) cudaFree(p);
    delete s;
    return KGB_OK;
}

int kgb_solver_set_diagonal(kgb_solver* s, const float* p) {
    if (!s) return set_error(KGB_ERR_VALUE, "solver_set_diagonal: null solver");
    if (p && !s->mvp) KGB_CUDA_TRY(cudaMalloc(&s->mvp, (size_t)s->n * sizeof(float)));
    if (p != s->pdiag) {
        // the captured iteration bakes the operator in
        if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
        if (s->graph) { cudaGraphDestroy(s->graph); s->graph = nullptr; }
    }
    s->pdiag = p;
    s->setup_done = false;
    return KGB_OK;
}

int kgb_solver_setup(kgb_solver* s, const float* y, const float* x0, const double* params, int nparams,
                     void* stream_) {
    if (!s || !y) return set_error(KGB_ERR_VALUE, "solver_setup: null pointer");
    cudaStream_t stream = (cudaStream_t)stream_;
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    int niter_setup = 10;
    if (s->kind == 1) { p[1] = 1e-8; p[2] = 1e-8; p[3] = 1e8; } else { p[1] = 1e-4; }
    for (int i = 0; i < nparams && i < 4; ++i) p[i] = params[i];
    if (nparams >= 5) niter_setup = (int)params[4];
    const int gn = grid_for(s->n), gm = grid_for(s->m);
    double* P0 = s->partials;
    double* P1 = s->partials + kRedBlocks;
    double* P2 = s->partials + 2 * kRedBlocks;
    int rc;
    init_state_kernel<<<1, 1, 0, stream>>>(s->st, s->kind, niter_setup, p[0], p[1], p[2], p[3]);
    if (s->kind == 1) {
        // x = x0 or 0; u = y - K x0 or y (cls_basic.py:944-956)
        if (x0) {
            KGB_CUDA_TRY(cudaMemcpyAsync(s->x, x0, s->n * 4, cudaMemcpyDeviceToDevice, stream));
            if ((rc = op_forward(s, x0, s->dv2, stream))) return rc;
            sub_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, y, s->dv2, s->m);
        } else {
            KGB_CUDA_TRY(cudaMemsetAsync(s->x, 0, s->n * 4, stream));
            KGB_CUDA_TRY(cudaMemcpyAsync(s->dv1, y, s->m * 4, cudaMemcpyDeviceToDevice, stream));
        }
        sq_partial_plain_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, s->m, P0);
        lsqr_setup_beta_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P0, gm);
        scale_by_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, s->m, s->st, 0);
        // v = K^H u when beta > 0, else v = x (cls_basic.py:957-969); computing
        // the adjoint unconditionally is harmless because it is discarded.
        if ((rc = op_adjoint(s, s->dv1, s->mv1, stream))) return rc;
        sq_partial_plain_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->n, P1);
        lsqr_setup_alfa_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P1, gn, s->cost);
        scale_by_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->n, s->st, 1);
        copy_if_beta_zero_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->x, s->n, s->st);  // v = x
        KGB_CUDA_TRY(cudaMemcpyAsync(s->mv2, s->mv1, s->n * 4, cudaMemcpyDeviceToDevice, stream));  // w = v
    } else {
        // CGLS setup (cls_basic.py:474-503)
        if (x0) {
            KGB_CUDA_TRY(cudaMemcpyAsync(s->x, x0, s->n * 4, cudaMemcpyDeviceToDevice, stream));
            if ((rc = op_forward(s, x0, s->dv2, stream))) return rc;
            sub_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, y, s->dv2, s->m);
            if ((rc = op_adjoint(s, s->dv1, s->mv1, stream))) return rc;
            axpy_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->x, (float)(-p[0]), s->n);  // unsquared damp
        } else {
            KGB_CUDA_TRY(cudaMemsetAsync(s->x, 0, s->n * 4, stream));
            KGB_CUDA_TRY(cudaMemcpyAsync(s->dv1, y, s->m * 4, cudaMemcpyDeviceToDevice, stream));
            if ((rc = op_adjoint(s, s->dv1, s->mv1, stream))) return rc;
        }
        if ((rc = op_forward(s, s->mv1, s->dv2, stream))) return rc;  // q = K c
        sq_partial_plain_kernel<<<gn, kRedThreads, 0, stream>>>(s->mv1, s->n, P0);
        sq_partial_plain_kernel<<<gm, kRedThreads, 0, stream>>>(s->dv1, s->m, P1);
        sq_partial_plain_kernel<<<gn, kRedThreads, 0, stream>>>(s->x, s->n, P2);
        cgls_setup_kernel<<<1, kRedThreads, 0, stream>>>(s->st, P0, gn, P1, gm, P2, gn, s->cost, s->cost1);
    }
    KGB_CUDA_TRY(cudaGetLastError());
    s->setup_done = true;
    return KGB_OK;
}

int kgb_solver_run(kgb_solver* s, int niter, int use_graph, void* stream_) {
    if (!s) return set_error(KGB_ERR_VALUE, "solver_run: null solver");
    if (!s->setup_done) return set_error(KGB_ERR_STATE, "solver_run: setup not called");
    if (niter <= 0) return KGB_OK;
    cudaStream_t stream = (cudaStream_t)stream_;
    // make room for the cost history of the iterations to come
    SolverState hst;
    KGB_CUDA_TRY(cudaMemcpyAsync(&hst, s->st, sizeof(SolverState), cudaMemcpyDeviceToHost, stream));
    KGB_CUDA_TRY(cudaStreamSynchronize(stream));
    int rc = ensure_cost(s, hst.iiter + niter + 2);
    if (rc) return rc;
    if (use_graph && stream != nullptr) {
        if ((rc = build_graph(s, stream))) return rc;
        set_target_kernel<<<1, 1, 0, stream>>>(s->st, niter, s->handle, 0);
        KGB_CUDA_TRY(cudaGetLastError());
        KGB_CUDA_TRY(cudaGraphLaunch(s->exec, stream));
        return KGB_OK;
    }
    set_target_kernel<<<1, 1, 0, stream>>>(s->st, niter, s->handle, 0);
    for (int k = 0; k < niter; ++k) {
        if ((rc = enqueue(s, stream, 0))) return rc;
        int active = 0;
        KGB_CUDA_TRY(cudaMemcpyAsync(&active, &s->st->active, sizeof(int), cudaMemcpyDeviceToHost, stream));
        KGB_CUDA_TRY(cudaStreamSynchronize(stream));
        if (!active) break;
    }
    return KGB_OK;
}

int kgb_solver_result(kgb_solver* s, float* x, double* out16, double* cost_host, int cost_capacity, void* stream_) {
    if (!s) return set_error(KGB_ERR_VALUE, "solver_result: null solver");
    cudaStream_t stream = (cudaStream_t)stream_;
    SolverState h;
    KGB_CUDA_TRY(cudaMemcpyAsync(&h, s->st, sizeof(SolverState), cudaMemcpyDeviceToHost, stream));
    if (x) KGB_CUDA_TRY(cudaMemcpyAsync(x, s->x, s->n * 4, cudaMemcpyDeviceToDevice, stream));
    KGB_CUDA_TRY(cudaStreamSynchronize(stream));
    if (out16) {
        for (int i = 0; i < 16; ++i) out16[i] = 0.0;
        out16[0] = h.iiter;
        if (s->kind == 1) {
            out16[1] = h.istop; out16[2] = h.r1norm; out16[3] = h.r2norm; out16[4] = h.anorm;
            out16[5] = h.acond; out16[6] = h.arnorm; out16[7] = h.xnorm; out16[8] = h.var_scalar;
        } else {
            out16[1] = h.kold < h.tol ? 1 : 2;  // cls_basic.py:625
            out16[9] = h.kold;
        }
    }
    if (cost_host && cost_capacity > 0) {
        const int n = std::min(cost_capacity, h.iiter + 1);
        KGB_CUDA_TRY(cudaMemcpy(cost_host, s->cost, n * sizeof(double), cudaMemcpyDeviceToHost));
        if (s->kind == 0 && cost_capacity >= 2 * n) {
            KGB_CUDA_TRY(cudaMemcpy(cost_host + n, s->cost1, n * sizeof(double), cudaMemcpyDeviceToHost));
        }
    }
    return KGB_OK;
}

}  // extern "C"
