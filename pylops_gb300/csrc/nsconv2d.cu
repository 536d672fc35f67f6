// 2-D non-stationary convolution (pylops/signalprocessing/nonstatconvolve2d.py:
// 121-300): a compact filter hs[ihx][ihz] (hx x hz, odd sizes) is given on a
// regular coarse grid of image points (ohx + k dhx, ohz + l dhz); the filter
// at image point (ix, iz) is the bilinear interpolation of its four
// neighbours (outside the coarse grid: the edge filter with weights 1/2,
// 1/2), and
//   forward  y[ix + a - hx/2][iz + b - hz/2] += x[ix][iz] h_(ix,iz)[a][b]
//   adjoint  y[ix][iz] = sum_ab h_(ix,iz)[a][b] x[ix + a - hx/2][iz + b - hz/2]
// inside the image.  Both directions run here as gathers: one thread per
// output point over the filter window, the input tile with its halo in
// shared memory, so there are no atomics and the result is deterministic.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "kgb_internal.h"

namespace kgb {
namespace nsc {

constexpr int TX = 16, TZ = 16;  // output tile (x rows, z columns)

// interpolation along one axis: filter indices (lo, hi) and weights
struct Interp {
    int lo, hi;
    float wlo, whi;
};

__device__ __forceinline__ Interp interp(int i, double o, double d, int n) {
    const double u = (i - o) / d;
    int l = (int)floor(u);
    Interp r;
    if (l < 0) {
        r.lo = r.hi = 0;
        r.wlo = r.whi = 0.5f;
    } else if (l >= n - 1) {
        r.lo = r.hi = n - 1;
        r.wlo = r.whi = 0.5f;
    } else {
        const double f = u - l;
        r.lo = l;
        r.hi = l + 1;
        r.whi = (float)f;
        r.wlo = (float)(1.0 - f);
    }
    return r;
}

template <bool ADJ>
__global__ void __launch_bounds__(TX * TZ)
nsconv2d_kernel(const float* __restrict__ x, float* __restrict__ y, const float* __restrict__ hs, int nx, int nz,
                int nhx, int nhz, int hx, int hz, double ohx, double ohz, double dhx, double dhz) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int hx2 = hx / 2, hz2 = hz / 2;
    const int SX = TX + hx - 1, SZ = TZ + hz - 1;  // tile + halo
    float* xs = reinterpret_cast<float*>(smem);
    Interp* ix_tab = reinterpret_cast<Interp*>(xs + (size_t)SX * SZ);
    Interp* iz_tab = ix_tab + SX;
    const int ox0 = blockIdx.x * TX, oz0 = blockIdx.y * TZ;
    const int tid = threadIdx.x;
    for (int k = tid; k < SX * SZ; k += blockDim.x) {
        const int a = k / SZ, b = k - a * SZ;
        const int gx = ox0 - hx2 + a, gz = oz0 - hz2 + b;
        xs[k] = (gx >= 0 && gx < nx && gz >= 0 && gz < nz) ? __ldg(x + (size_t)gx * nz + gz) : 0.f;
    }
    if (!ADJ) {  // the forward needs the filter of every source point of the tile
        for (int k = tid; k < SX; k += blockDim.x) ix_tab[k] = interp(ox0 - hx2 + k, ohx, dhx, nhx);
        for (int k = tid; k < SZ; k += blockDim.x) iz_tab[k] = interp(oz0 - hz2 + k, ohz, dhz, nhz);
    }
    __syncthreads();
    const int tz = tid % TZ, tx = tid / TZ;  // z fastest: coalesced output rows
    const int ox = ox0 + tx, oz = oz0 + tz;
    if (ox >= nx || oz >= nz) return;
    const size_t fsz = (size_t)hx * hz;
    float acc = 0.f;
    if (ADJ) {
        const Interp px = interp(ox, ohx, dhx, nhx), pz = interp(oz, ohz, dhz, nhz);
        const float* f_tl = hs + ((size_t)px.lo * nhz + pz.lo) * fsz;
        const float* f_bl = hs + ((size_t)px.lo * nhz + pz.hi) * fsz;
        const float* f_tr = hs + ((size_t)px.hi * nhz + pz.lo) * fsz;
        const float* f_br = hs + ((size_t)px.hi * nhz + pz.hi) * fsz;
        const float w_tl = pz.wlo * px.wlo, w_bl = pz.whi * px.wlo, w_tr = pz.wlo * px.whi, w_br = pz.whi * px.whi;
        for (int a = 0; a < hx; ++a) {
            const float* xrow = xs + (size_t)(tx + a) * SZ + tz;
            const size_t fa = (size_t)a * hz;
            for (int b = 0; b < hz; ++b) {
                const float h = w_tl * __ldg(f_tl + fa + b) + w_bl * __ldg(f_bl + fa + b) +
                                w_tr * __ldg(f_tr + fa + b) + w_br * __ldg(f_br + fa + b);
                acc = fmaf(h, xrow[b], acc);
            }
        }
    } else {
        // source point (ox - a + hx2, oz - b + hz2) contributes x h_src[a][b];
        // in tile coordinates its row is tx + hx - 1 - a, its column tz + hz - 1 - b
        for (int a = 0; a < hx; ++a) {
            const int sr = tx + hx - 1 - a;
            const Interp px = ix_tab[sr];
            const float* xrow = xs + (size_t)sr * SZ;
            const size_t fa = (size_t)a * hz;
            const float* fl = hs + (size_t)px.lo * nhz * fsz + fa;
            const float* fh = hs + (size_t)px.hi * nhz * fsz + fa;
            for (int b = 0; b < hz; ++b) {
                const int sc = tz + hz - 1 - b;
                const float xv = xrow[sc];
                if (xv == 0.f) continue;
                const Interp pz = iz_tab[sc];
                const float h = pz.wlo * (px.wlo * __ldg(fl + (size_t)pz.lo * fsz + b) +
                                          px.whi * __ldg(fh + (size_t)pz.lo * fsz + b)) +
                                pz.whi * (px.wlo * __ldg(fl + (size_t)pz.hi * fsz + b) +
                                          px.whi * __ldg(fh + (size_t)pz.hi * fsz + b));
                acc = fmaf(xv, h, acc);
            }
        }
    }
    y[(size_t)ox * nz + oz] = acc;
}

}  // namespace nsc
}  // namespace kgb

using namespace kgb;

extern "C" int kgb_nsconv2d_apply(const float* x, float* y, const float* hs, int nx, int nz, int nhx, int nhz, int hx,
                                  int hz, double ohx, double ohz, double dhx, double dhz, int adjoint, void* stream) {
    if (!x || !y || !hs) return set_error(KGB_ERR_VALUE, "nsconv2d: null pointer");
    if (nx <= 0 || nz <= 0 || nhx <= 0 || nhz <= 0 || hx <= 0 || hz <= 0)
        return set_error(KGB_ERR_VALUE, "nsconv2d: sizes must be positive");
    if (hx % 2 == 0 || hz % 2 == 0) return set_error(KGB_ERR_VALUE, "filters hs must have odd length");
    if (!(dhx > 0) || !(dhz > 0)) return set_error(KGB_ERR_VALUE, "nsconv2d: filter grid steps must be positive");
    const size_t SX = nsc::TX + hx - 1, SZ = nsc::TZ + hz - 1;
    const size_t smem = SX * SZ * sizeof(float) + (SX + SZ) * sizeof(nsc::Interp);
    if (smem > 227 * 1024) return set_error(KGB_ERR_NOT_IMPLEMENTED, "nsconv2d: filter %dx%d too large", hx, hz);
    dim3 grid((unsigned)((nx + nsc::TX - 1) / nsc::TX), (unsigned)((nz + nsc::TZ - 1) / nsc::TZ));
    cudaStream_t s = (cudaStream_t)stream;
    if (adjoint) {
        auto k = nsc::nsconv2d_kernel<true>;
        KGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, nsc::TX * nsc::TZ, smem, s>>>(x, y, hs, nx, nz, nhx, nhz, hx, hz, ohx, ohz, dhx, dhz);
    } else {
        auto k = nsc::nsconv2d_kernel<false>;
        KGB_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k<<<grid, nsc::TX * nsc::TZ, smem, s>>>(x, y, hs, nx, nz, nhx, nhz, hx, hz, ohx, ohz, dhx, dhz);
    }
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}
