// BF16 "TN" GEMM on the 5th-generation tensor cores (tcgen05) for sm_103a:
//   C[m][n] = sum_k A[m][k] * B[n][k]  (+ bias[n], optional ReLU)
// A (M x K) and B (N x K) are row-major bf16 with K contiguous; C is float32
// or bf16 with leading dimension ldc.  This is the one tensor-core kernel of
// the U-Net preconditioner: its convolutions (forward, data gradient, weight
// gradient) are lowered to it through im2col / transposes.
//
// Structure (persistent: one CTA per SM walking 128 x BN output tiles, 6 warps):
//  * warp 0, one lane: TMA producer -- 2-D tiled bulk-tensor loads of the A
//    and B k-tiles (64 bf16 = 128 bytes along K) with 128-byte swizzle into a
//    shared-memory ring of up to 8 stages, completion counted on "full"
//    mbarriers, running ahead across tile boundaries;
//  * warp 1: allocates and frees tensor memory (two BN-column accumulators);
//    one lane issues the MMAs -- four tcgen05.mma (K = 16 each) per k-tile on
//    shared-memory descriptors; tcgen05.commit releases the stage ("empty"
//    mbarrier) and, after a tile's last k-tile, hands its accumulator to the
//    epilogue;
//  * warps 2-5: epilogue -- tcgen05.ld of their 32 accumulator lanes, bias /
//    ReLU, store, then hand the accumulator back to the MMA warp, so that one
//    tile's epilogue overlaps the next tile's MMAs.
// Every mbarrier wait is bounded: after ~2^26 polls the CTA records an error
// code in `err`, waits (bounded) for its copies and MMAs in flight, frees
// tensor memory and leaves.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kgb_internal.h"

namespace kgb {
namespace {

constexpr int BM = 128;
constexpr int BK = 64;          // bf16 elements per k-tile row = 128 bytes (one swizzle atom)
constexpr uint32_t kSpinLimit = 1u << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// bounded wait on the phase with parity `parity`; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\n"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            "selp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(dst), "l"(map), "r"(bar), "r"(c0), "r"(c1)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1,
                                            int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];"
        ::"r"(dst), "l"(map), "r"(bar), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}

// 4-D tiled load (implicit convolution: channels, width, height, image).
// Coordinates other than the innermost may be negative or past the end: the
// box is zero-filled there (the convolution's padding).
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int c0, int c1,
                                            int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5, %6}], [%2];"
        ::"r"(dst), "l"(map), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
        : "memory");
}

// Geometry of an implicit 3x3 stride-1 convolution over NHWC bf16 input:
// an M tile of 128 output pixels is a box of bh rows x bw columns of one
// image; k-tile g is (tap = g / cblk, channel block g % cblk) and reads the
// input shifted by sgn * (ky - 1, kx - 1) (sgn = -1: the transposed
// convolution of the data gradient).  Weight gradient: cblk = 128-row tiles
// per ky (rows of A are (ky, kx, channel)), k-tile = 64 pixels of one image
// row.
struct ConvGeom {
    int H, W, cblk, sgn;
    int nimg;  // weight gradient: images per shifted copy
};

// Operand modes of the GEMM kernel: plain 2-D A; implicit 3x3 convolution
// (A from shifted 4-D boxes of NHWC activations); weight gradient of a 3x3
// convolution (A from the column-shifted channel-major copies, see
// kgb_conv3x3_wgrad_bf16).
constexpr int kModePlain = 0, kModeConv = 1, kModeWgrad = 2;

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle.
// start address >> 4 in bits [0,14); leading byte offset (unused for
// swizzled K-major, 1) in [16,30); stride byte offset = 1024 B between
// 8-row groups, >> 4, in [32,46); descriptor version 1 in [46,48); layout
// SWIZZLE_128B = 2 in [61,64).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Instruction descriptor, kind::f16: D f32 (bits [4,6) = 1), A and B bf16
// (bits [7,10) and [10,13) = 1), both K-major, N >> 3 in [17,23), M >> 4 in
// [24,29).
__host__ __device__ constexpr uint32_t idesc_bf16(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Shared-memory ring depth: as many stages as fit in ~192 KB (one CTA per SM).
template <int BN>
__host__ __device__ constexpr int gemm_stages() {
    return (192 * 1024) / (BM * BK * 2 + BN * BK * 2) < 8 ? (192 * 1024) / (BM * BK * 2 + BN * BK * 2) : 8;
}

constexpr int kGemmThreads = 192;  // warp 0 producer, warp 1 MMA, warps 2-5 epilogue

// Epilogue of one 128 x BN tile: the calling warp reads tensor-memory lanes
// 32 q .. 32 q + 31 of accumulator a (rows m0 + 32 q + lane), adds the bias,
// applies ReLU (flags & 1) and stores float32 or bf16 (flags & 2; 16-byte
// vector stores when flags & 4).
template <int BN>
__device__ __forceinline__ void epilogue_store(uint32_t tmem, int q, int a, int lane, int m0, int n0, int M, int N,
                                               int ldc, void* Cz, const float* __restrict__ bias, int flags) {
    const int row = m0 + q * 32 + lane;
    for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * BN + c0);
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
              "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
              "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
              "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (row < M && (flags & 4) && n0 + c0 + 32 <= N) {
            // whole 32-column chunk, 16-byte aligned row segment
            float v[32];
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
                v[jj] = __uint_as_float(r[jj]);
                if (bias) v[jj] += __ldg(bias + n0 + c0 + jj);
                if (flags & 1) v[jj] = fmaxf(v[jj], 0.f);
            }
            if (flags & 2) {
                uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(Cz) + (size_t)row * ldc +
                                                      n0 + c0);
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    uint4 w4;
                    w4.x = pack_bf16(v[8 * qq + 0], v[8 * qq + 1]);
                    w4.y = pack_bf16(v[8 * qq + 2], v[8 * qq + 3]);
                    w4.z = pack_bf16(v[8 * qq + 4], v[8 * qq + 5]);
                    w4.w = pack_bf16(v[8 * qq + 6], v[8 * qq + 7]);
                    dst[qq] = w4;
                }
            } else {
                float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(Cz) + (size_t)row * ldc + n0 +
                                                        c0);
#pragma unroll
                for (int qq = 0; qq < 8; ++qq)
                    dst[qq] = make_float4(v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3]);
            }
        } else if (row < M) {
#pragma unroll
            for (int jj = 0; jj < 32; ++jj) {
                const int col = n0 + c0 + jj;
                if (col < N) {
                    float v = __uint_as_float(r[jj]);
                    if (bias) v += __ldg(bias + col);
                    if (flags & 1) v = fmaxf(v, 0.f);
                    if (flags & 2)
                        reinterpret_cast<__nv_bfloat16*>(Cz)[(size_t)row * ldc + col] = __float2bfloat16(v);
                    else
                        reinterpret_cast<float*>(Cz)[(size_t)row * ldc + col] = v;
                }
            }
        }
    }
}

// Persistent GEMM: each CTA walks output tiles t = blockIdx.x, + gridDim.x,
// ... (tile t: n tile t % tiles_n, m tile (t / tiles_n) % tiles_m, k split
// t / (tiles_n tiles_m)), so the tiles that run together share their A rows
// in L2.  The producer streams the k-tiles of consecutive tiles through one
// ring without draining it between tiles; the accumulator is double-buffered
// in tensor memory (2 x BN columns), so the MMAs of tile j + 1 run while the
// epilogue warps read tile j.
template <int BN, int MODE>
__global__ void __launch_bounds__(kGemmThreads, 1)
gemm_tn_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, void* __restrict__ C,
               int M, int N, int K, int ldc, const float* __restrict__ bias, int flags, int* __restrict__ err,
               int kt_per, int64_t split_stride, const ConvGeom cg, int tiles_m, int tiles_n, int splits) {
    constexpr int S = gemm_stages<BN>();
    constexpr int A_BYTES = BM * BK * 2;
    constexpr int B_BYTES = BN * BK * 2;
    extern __shared__ uint8_t smem_dyn[];
    // 1024-byte alignment for the swizzled tiles
    const uint32_t base_s = smem_u32(smem_dyn);
    const uint32_t pad = (1024 - (base_s & 1023)) & 1023;
    uint8_t* smem = smem_dyn + pad;
    const uint32_t sA = smem_u32(smem);
    const uint32_t sB = sA + S * A_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * (A_BYTES + B_BYTES));
    // bars: [0, S) full, [S, 2S) empty, then accumulator full x2, accumulator
    // empty x2, drain; then the tmem slot and an abort flag
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 5);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const uint32_t bar_full = smem_u32(bars);
    const uint32_t bar_empty = bar_full + 8 * S;
    const uint32_t bar_tfull = bar_full + 16 * S;
    const uint32_t bar_tempty = bar_tfull + 16;
    const uint32_t bar_drain = bar_tempty + 16;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ktiles_total = (K + BK - 1) / BK;
    const int ntiles = tiles_m * tiles_n * splits;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(bar_tfull + 8 * a, 1);
            mbar_init(bar_tempty + 8 * a, 4);  // one arrival per epilogue warp
        }
        mbar_init(bar_drain, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)(2 * BN)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // producer: k-tiles of this CTA's tiles in order, `it` counting them
            uint32_t it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int tn = t % tiles_n, rest = t / tiles_n;
                const int m0 = (rest % tiles_m) * BM, n0 = tn * BN, z = rest / tiles_m;
                const int kt0 = z * kt_per;
                const int nkt = min(ktiles_total - kt0, kt_per);
                int img = 0, h0 = 0, w0 = 0;
                if (MODE == kModeConv) {
                    const int hw = cg.H * cg.W;
                    img = m0 / hw;
                    const int r = m0 - img * hw;
                    h0 = r / cg.W;
                    w0 = r - h0 * cg.W;
                }
                for (int kt = 0; kt < nkt; ++kt, ++it) {
                    const int s = (int)(it % S);
                    if ((it >= (uint32_t)S && !mbar_wait(bar_empty + 8 * s, ((it / S) - 1) & 1)) || *abort_flag) {
                        ok = false;
                        break;
                    }
                    if (MODE == kModeWgrad) {
                        // 64 pixels of one image row; the A tile is rows
                        // j0 .. j0 + 127 of the 3 C rows (kx, c) of image row
                        // h + ky - 1 (zero fill outside the image and past 3 C)
                        const int p0 = (kt0 + kt) * BK;
                        const int hw = cg.H * cg.W;
                        const int b = p0 / hw, r = p0 - b * hw;
                        const int h = r / cg.W, wp = r - h * cg.W;
                        const int tm = m0 / BM;
                        const int ky = tm / cg.cblk, j0 = (tm - ky * cg.cblk) * BM;
                        mbar_expect_tx(bar_full + 8 * s, A_BYTES + B_BYTES);
                        tma_load_4d(sA + s * A_BYTES, &tmA, bar_full + 8 * s, wp, j0, h + ky - 1, b);
                        tma_load_3d(sB + s * B_BYTES, &tmB, bar_full + 8 * s, wp, n0, b * cg.H + h);
                        continue;
                    }
                    mbar_expect_tx(bar_full + 8 * s, A_BYTES + B_BYTES);
                    if (MODE == kModeConv) {
                        const int g = kt0 + kt;
                        const int tap = g / cg.cblk, cb = g - tap * cg.cblk;
                        const int ky = tap / 3, kx = tap - ky * 3;
                        tma_load_4d(sA + s * A_BYTES, &tmA, bar_full + 8 * s, cb * BK, w0 + cg.sgn * (kx - 1),
                                    h0 + cg.sgn * (ky - 1), img);
                    } else {
                        tma_load_2d(sA + s * A_BYTES, &tmA, bar_full + 8 * s, (kt0 + kt) * BK, m0);
                    }
                    tma_load_2d(sB + s * B_BYTES, &tmB, bar_full + 8 * s, (kt0 + kt) * BK, n0);
                }
            }
            if (!ok) *abort_flag = 1;
            // the copies issued last (at most S stages) land before the CTA
            // can leave: wait for their full phases (already complete on the
            // normal path)
            for (uint32_t j = it > (uint32_t)S ? it - S : 0u; j < it; ++j)
                mbar_wait(bar_full + 8 * (j % S), (j / S) & 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // MMA issuer
            constexpr uint32_t idesc = idesc_bf16(BM, BN);
            uint32_t it = 0;
            bool ok = true;
            int j = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++j) {
                const int a = j & 1, u = j >> 1;
                // accumulator a is free once the epilogue has read tile j - 2
                if (j >= 2 && !mbar_wait(bar_tempty + 8 * a, (u - 1) & 1)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const int z = (t / tiles_n) / tiles_m;
                const int nkt = min(ktiles_total - z * kt_per, kt_per);
                const uint32_t dacc = tmem + (uint32_t)(a * BN);
                for (int kt = 0; kt < nkt; ++kt, ++it) {
                    const int s = (int)(it % S);
                    if (!mbar_wait(bar_full + 8 * s, (it / S) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k) {
                        const uint64_t da = sw128_desc(sA + s * A_BYTES + k * 32);
                        const uint64_t db = sw128_desc(sB + s * B_BYTES + k * 32);
                        const uint32_t acc = (kt > 0 || k > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                            ::"r"(dacc), "l"(da), "l"(db), "r"(idesc), "r"(acc));
                    }
                    // release the stage when these MMAs have read it
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                                 ::"r"(bar_empty + 8 * s) : "memory");
                }
                if (!ok) break;
                // accumulator a holds tile t when these MMAs complete
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             ::"r"(bar_tfull + 8 * a) : "memory");
            }
            if (!ok) *abort_flag = 1;
            // every MMA issued completes before tensor memory is freed
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(bar_drain) : "memory");
            mbar_wait(bar_drain, 0);
        }
    } else {
        // epilogue: warp w reads tensor-memory lanes 32 (w % 4) .. + 31,
        // i.e. rows m0 + 32 (w % 4) + lane of each tile
        const int q = warp & 3;
        int j = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++j) {
            const int a = j & 1, u = j >> 1;
            const bool ready = __all_sync(0xffffffffu, mbar_wait(bar_tfull + 8 * a, u & 1));
            if (!ready || *abort_flag) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int tn = t % tiles_n, rest = t / tiles_n;
            const int m0 = (rest % tiles_m) * BM, n0 = tn * BN, z = rest / tiles_m;
            void* Cz = z ? reinterpret_cast<void*>(reinterpret_cast<float*>(C) + z * split_stride) : C;
            epilogue_store<BN>(tmem, q, a, lane, m0, n0, M, N, ldc, Cz, bias, flags);
            // this warp's lanes of accumulator a are read: hand it back
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar_tempty + 8 * a) : "memory");
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag && err) atomicExch(err, 1);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * BN)));
    }
}

// Implicit convolutions with resident weights: tiles are 128 consecutive
// pixels of the source grid (the grid the A operand is read from), either
// part of one row (width a multiple of 128) or 128 / W whole rows (W
// dividing 128).  A plan lists, per channel block, up to four boxes of 64
// channels each -- the box of entry h starts at source row i + row_dh[h],
// column w0 + row_dc[h] (zero fill outside the image) -- and per box up to
// three taps: the A operand of a tap is that box starting `off` 128-byte rows
// in (the descriptor's 128-byte swizzle follows the absolute shared-memory
// address, so a start offset by whole rows reads the rows the TMA wrote
// there), its B operand the weight tile of kernel tap `w`.  Row tiles use
// halo boxes (136 pixels of one row, shared by the taps of one kernel row);
// multi-row tiles use one box of the tile's own shape per tap.  The weights
// of all 9 taps (N <= BN rows) stay in shared memory for the whole kernel.
// Output pixel of source pixel (img, i, j): (img, out_rs i + out_rb, out_cs j
// + out_cb) of an Hout x Wout image; the 32 rows of one epilogue warp lie in
// one source row (W a multiple of 32), so they are out_cs pixels apart.
// Plans: the 3x3 stride-1 convolution and its transposed form (3 halo rows,
// 3 taps each), and the four pixel-parity classes of the data gradient of a
// 3x3 stride-2 convolution (1, 2, 2 or 4 taps, outputs 2 pixels apart).
// Same persistence, accumulator double-buffering, epilogue and bounded
// waits as gemm_tn_kernel.
constexpr int kHaloRows = 136;                  // 130 needed, 8-row multiple
constexpr int kHaloBytes = 18 * 1024;           // 136 x 128 B, rounded to 1 KB
constexpr int kHaloMaxStages = 8;

constexpr int kPlanBoxes = 4;

struct HaloPlan {
    int nrows;                     // boxes per channel block (1..4)
    int row_dh[kPlanBoxes];        // source row offset of each box
    int row_dc[kPlanBoxes];        // source column offset of each box, relative to the tile's
    int row_ntaps[kPlanBoxes];     // taps per box (1..3)
    int tap_off[kPlanBoxes][3], tap_w[kPlanBoxes][3];  // per box and tap: row offset in the box, kernel tap
    int box_bytes;                 // bytes of one box
    int out_rs, out_rb, out_cs, out_cb, Hout, Wout;
    int ksteps_last;               // 16-channel k-steps of the last channel block that hold channels
};

template <int BN>
__global__ void __launch_bounds__(kGemmThreads, 1)
conv_halo_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmW, void* __restrict__ C,
                 int M, int N, const float* __restrict__ bias, int flags, int* __restrict__ err, const ConvGeom cg,
                 const __grid_constant__ HaloPlan plan, int stages) {
    constexpr int W_TILE = BN * BK * 2;  // one (tap, channel block) weight tile
    const int S = stages;
    const int nw = 9 * cg.cblk;          // resident weight tiles
    extern __shared__ uint8_t smem_dyn[];
    const uint32_t base_s = smem_u32(smem_dyn);
    const uint32_t pad = (1024 - (base_s & 1023)) & 1023;
    uint8_t* smem = smem_dyn + pad;
    const uint32_t sW = smem_u32(smem);
    const uint32_t sR = sW + nw * W_TILE;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + nw * W_TILE + S * kHaloBytes);
    // bars: [0, S) full, [S, 2S) empty, accumulator full x2, empty x2,
    // drain, weights; then the tmem slot and an abort flag
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 6);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const uint32_t bar_full = smem_u32(bars);
    const uint32_t bar_empty = bar_full + 8 * S;
    const uint32_t bar_tfull = bar_full + 16 * S;
    const uint32_t bar_tempty = bar_tfull + 16;
    const uint32_t bar_drain = bar_tempty + 16;
    const uint32_t bar_w = bar_drain + 8;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = M / BM;
    const int steps = plan.nrows * cg.cblk;  // halo rows per tile
    const int hw = cg.H * cg.W;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(bar_tfull + 8 * a, 1);
            mbar_init(bar_tempty + 8 * a, 4);
        }
        mbar_init(bar_drain, 1);
        mbar_init(bar_w, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)(2 * BN)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // the weights: tile g = tap * cblk + cb is columns g * 64 .. + 63
            mbar_expect_tx(bar_w, (uint32_t)(nw * W_TILE));
            for (int g = 0; g < nw; ++g) tma_load_2d(sW + g * W_TILE, &tmW, bar_w, g * BK, 0);
            uint32_t it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                const int m0 = t * BM;
                const int img = m0 / hw, r = m0 - img * hw;
                const int h = r / cg.W, w0 = r - h * cg.W;
                for (int st = 0; st < steps; ++st, ++it) {
                    const int s = (int)(it % S);
                    if ((it >= (uint32_t)S && !mbar_wait(bar_empty + 8 * s, ((it / S) - 1) & 1)) || *abort_flag) {
                        ok = false;
                        break;
                    }
                    const int cb = st / plan.nrows, hr = st - cb * plan.nrows;
                    mbar_expect_tx(bar_full + 8 * s, (uint32_t)plan.box_bytes);
                    tma_load_4d(sR + s * kHaloBytes, &tmX, bar_full + 8 * s, cb * BK, w0 + plan.row_dc[hr],
                                h + plan.row_dh[hr], img);
                }
            }
            if (!ok) *abort_flag = 1;
            for (uint32_t j = it > (uint32_t)S ? it - S : 0u; j < it; ++j)
                mbar_wait(bar_full + 8 * (j % S), (j / S) & 1);
            mbar_wait(bar_w, 0);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(BM, BN);
            bool ok = mbar_wait(bar_w, 0);
            uint32_t it = 0;
            int j = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++j) {
                const int a = j & 1, u = j >> 1;
                if (j >= 2 && !mbar_wait(bar_tempty + 8 * a, (u - 1) & 1)) {
                    ok = false;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t dacc = tmem + (uint32_t)(a * BN);
                for (int st = 0; st < steps; ++st, ++it) {
                    const int s = (int)(it % S);
                    if (!mbar_wait(bar_full + 8 * s, (it / S) & 1)) {
                        ok = false;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const int cb = st / plan.nrows, hr = st - cb * plan.nrows;
                    const int nk = cb == cg.cblk - 1 ? plan.ksteps_last : BK / 16;
                    const uint32_t halo = sR + s * kHaloBytes;
                    for (int q = 0; q < plan.row_ntaps[hr]; ++q) {
                        const int off = plan.tap_off[hr][q];
                        const uint32_t wt = sW + (plan.tap_w[hr][q] * cg.cblk + cb) * W_TILE;
#pragma unroll
                        for (int k = 0; k < BK / 16; ++k) {
                            if (k >= nk) break;  // zero-filled channels past C contribute nothing
                            const uint64_t da = sw128_desc(halo + off * 128 + k * 32);
                            const uint64_t db = sw128_desc(wt + k * 32);
                            const uint32_t acc = (st > 0 || q > 0 || k > 0) ? 1u : 0u;
                            asm volatile(
                                "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                                ::"r"(dacc), "l"(da), "l"(db), "r"(idesc), "r"(acc));
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                                 ::"r"(bar_empty + 8 * s) : "memory");
                }
                if (!ok) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             ::"r"(bar_tfull + 8 * a) : "memory");
            }
            if (!ok) *abort_flag = 1;
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(bar_drain) : "memory");
            mbar_wait(bar_drain, 0);
        }
    } else {
        const int q = warp & 3;
        int j = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++j) {
            const int a = j & 1, u = j >> 1;
            const bool ready = __all_sync(0xffffffffu, mbar_wait(bar_tfull + 8 * a, u & 1));
            if (!ready || *abort_flag) {
                *abort_flag = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // this warp's 32 rows: one source row segment, outputs out_cs
            // apart; `opix` is the output pixel of tile row 0 on that line
            // (tile rows q * 32 + lane), at least 0 since the output index
            // grows with the source pixel
            const int m0 = t * BM;
            const int img = m0 / hw, p = m0 - img * hw + q * 32;
            const int hq = p / cg.W, wq = p - hq * cg.W;
            const int64_t opix = ((int64_t)img * plan.Hout + (int64_t)plan.out_rs * hq + plan.out_rb) * plan.Wout +
                                 (int64_t)plan.out_cs * wq + plan.out_cb - (int64_t)plan.out_cs * (q * 32);
            void* Ct = (flags & 2) ? static_cast<void*>(reinterpret_cast<__nv_bfloat16*>(C) + opix * N)
                                   : static_cast<void*>(reinterpret_cast<float*>(C) + opix * N);
            epilogue_store<BN>(tmem, q, a, lane, 0, 0, BM, N, plan.out_cs * N, Ct, bias, flags);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar_tempty + 8 * a) : "memory");
        }
    }
    __syncwarp();
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0 && *abort_flag && err) atomicExch(err, 1);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)(2 * BN)));
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// rows x cols bf16 matrix, row stride ld elements, box = box_rows x 64
int make_map(CUtensorMap* map, const void* base, int64_t rows, int64_t cols, int64_t ld, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(KGB_ERR_CUDA, "gemm: cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KGB_ERR_VALUE, "gemm: tensor map rejected (CUresult %d)", (int)r);
    return KGB_OK;
}

// NHWC bf16 activations (B images of H x W pixels, C channels) as a 4-D
// tensor {C, W, H, B}; box {64 channels, bw, bh, 1} = 128 pixels of one
// image, each a 128-byte row of the shared-memory tile (the layout of the
// 2-D A tile).
int make_map_nhwc(CUtensorMap* map, const void* base, int B, int H, int W, int C, int bw, int bh) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(KGB_ERR_CUDA, "conv: cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)bw, (cuuint32_t)bh, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KGB_ERR_VALUE, "conv: tensor map rejected (CUresult %d)", (int)r);
    return KGB_OK;
}

// Column-shifted copies stacked per image row, xT3[b][h][kx][c][w] (bf16),
// as a 4-D tensor {W, 3C, H, B}; box {64 columns, 128 rows (kx, c), 1, 1} =
// one 128-row A tile (rows past 3 C are zero fill).
int make_map_wgrad(CUtensorMap* map, const void* base, int B, int H, int W, int C) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(KGB_ERR_CUDA, "wgrad: cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[4] = {(cuuint64_t)W, (cuuint64_t)3 * C, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {(cuuint64_t)W * 2, (cuuint64_t)3 * C * W * 2, (cuuint64_t)H * 3 * C * W * 2};
    cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)BM, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KGB_ERR_VALUE, "wgrad: tensor map rejected (CUresult %d)", (int)r);
    return KGB_OK;
}

// Row-blocked output gradient gTr[r][n][w] (bf16, r = b H + h) as a 3-D
// tensor {W, N, B H}; box {64 columns, box_rows gradients, 1}.
int make_map_rows(CUtensorMap* map, const void* base, int64_t R, int W, int N, int box_rows) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(KGB_ERR_CUDA, "wgrad: cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)N, (cuuint64_t)R};
    cuuint64_t strides[2] = {(cuuint64_t)W * 2, (cuuint64_t)N * W * 2};
    cuuint32_t box[3] = {(cuuint32_t)BK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KGB_ERR_VALUE, "wgrad: tensor map rejected (CUresult %d)", (int)r);
    return KGB_OK;
}

// dW[n][tap C + c] = sum over z of work[z][ky Mky + kx C + c][n] (tap = 3 ky
// + kx; Mky rows per ky), in order z = 0, 1, ...
__global__ void wgrad_sum_kernel(const float* __restrict__ work, float* __restrict__ dW, int M, int N, int splits,
                                 int C, int Mky, int ldw) {
    const int Q = 9 * C;
    const int64_t total = (int64_t)Q * N, mn = (int64_t)M * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int n = (int)(i / Q), q = (int)(i - (int64_t)n * Q);
        const int tap = q / C, c = q - tap * C;
        const int ky = tap / 3, kx = tap - ky * 3;
        const int64_t row = (int64_t)ky * Mky + kx * C + c;
        float acc = 0.f;
        for (int z = 0; z < splits; ++z) acc += work[z * mn + row * N + n];
        dW[(int64_t)n * ldw + q] = acc;
    }
}

// NHWC activations as the 4-D tensor {C, W, H, B} with a halo box {64
// channels, 136 pixels, 1, 1}.
int make_map_halo(CUtensorMap* map, const void* base, int B, int H, int W, int C) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return set_error(KGB_ERR_CUDA, "conv: cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[4] = {(cuuint64_t)C, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B};
    cuuint64_t strides[3] = {(cuuint64_t)C * 2, (cuuint64_t)W * C * 2, (cuuint64_t)H * W * C * 2};
    cuuint32_t box[4] = {(cuuint32_t)BK, (cuuint32_t)kHaloRows, 1, 1};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(KGB_ERR_VALUE, "conv: tensor map rejected (CUresult %d)", (int)r);
    return KGB_OK;
}

int sm_count();

constexpr size_t kSmemLimit = 227 * 1024;

// shared memory of conv_halo_kernel with `stages` halo rows
size_t halo_smem(int BN, int cblk, int stages) {
    return 1024 + (size_t)9 * cblk * BN * BK * 2 + (size_t)stages * kHaloBytes + 8 * (2 * stages + 6) + 16;
}

// halo rows that fit next to the resident weights (0 if fewer than 3)
int halo_stages(int BN, int cblk) {
    for (int st = kHaloMaxStages; st >= 3; --st)
        if (halo_smem(BN, cblk, st) <= kSmemLimit) return st;
    return 0;
}

template <int BN>
int halo_launch(const CUtensorMap& mx, const CUtensorMap& mw, void* y, int M, int N, const float* bias, int flags,
                int* err, const ConvGeom& cg, const HaloPlan& plan, int stages, cudaStream_t s) {
    const size_t smem = halo_smem(BN, cg.cblk, stages);
    KGB_CUDA_TRY(cudaFuncSetAttribute(conv_halo_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int ntiles = M / BM;
    const int grid = std::min(ntiles, sm_count());
    conv_halo_kernel<BN><<<grid, kGemmThreads, smem, s>>>(mx, mw, y, M, N, bias, flags, err, cg, plan, stages);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

// The 3x3 stride-1 convolution (sgn = +1) or its transposed form (sgn = -1):
// halo rows ky = 0, 1, 2 at source row offset sgn (ky - 1), columns from
// w0 - 1, taps kx at halo row offset kx (2 - kx transposed).
// k-steps of the last 64-channel block of C channels that hold channels
int last_ksteps(int C) {
    return (C - ((C - 1) / BK) * BK + 15) / 16;
}

HaloPlan plan_conv3x3(int sgn, int Hout, int Wout, int C) {
    HaloPlan p{};
    p.ksteps_last = last_ksteps(C);
    p.nrows = 3;
    p.box_bytes = kHaloRows * BK * 2;
    for (int ky = 0; ky < 3; ++ky) {
        p.row_dh[ky] = sgn * (ky - 1);
        p.row_dc[ky] = -1;
        p.row_ntaps[ky] = 3;
        for (int kx = 0; kx < 3; ++kx) {
            p.tap_off[ky][kx] = sgn > 0 ? kx : 2 - kx;
            p.tap_w[ky][kx] = ky * 3 + kx;
        }
    }
    p.out_rs = 1;
    p.out_rb = 0;
    p.out_cs = 1;
    p.out_cb = 0;
    p.Hout = Hout;
    p.Wout = Wout;
    return p;
}

// Data gradient of a 3x3 stride-2 convolution (padding 1), output pixels of
// parity (a, b): dx[2i + a][2j + b] = sum over the taps (ky, kx) with
// ky = 1 (a = 0) or ky in {0, 2} (a = 1), likewise kx, of W_tap^T g[i + di][j + dj],
// di = 1 for ky = 0 and 0 otherwise (dj likewise): the halo rows are g rows
// i + 1 and i, its columns start at j0, and a tap with dj = 1 starts one
// row into the halo.
// Class (a, b) of the data gradient of a 3x3 stride-2 convolution: input
// pixel (2i + a, 2j + b) collects gradient pixel (i + dy, j + dx) through
// kernel tap (ky, kx) for ky in {1} (a = 0) or {0, 2} (a = 1), dy = 1 for
// ky = 0 else 0, and the same along columns.  halo: row tiles, one halo box
// per kernel row shared by its column taps; otherwise one box per tap.
HaloPlan plan_s2_dgrad(int a, int b, int Hout, int Wout, int C, bool halo) {
    HaloPlan p{};
    p.ksteps_last = last_ksteps(C);
    const int kys[2] = {a == 0 ? 1 : 0, 2}, nky = a == 0 ? 1 : 2;
    const int kxs[2] = {b == 0 ? 1 : 0, 2}, nkx = b == 0 ? 1 : 2;
    p.nrows = halo ? nky : nky * nkx;
    p.box_bytes = (halo ? kHaloRows : BM) * BK * 2;
    for (int r = 0; r < nky; ++r) {
        const int ky = kys[r];
        for (int q = 0; q < nkx; ++q) {
            const int kx = kxs[q];
            const int e = halo ? r : r * nkx + q, t = halo ? q : 0;
            p.row_dh[e] = ky == 0 ? 1 : 0;
            p.row_dc[e] = halo ? 0 : (kx == 0 ? 1 : 0);
            p.row_ntaps[e] = halo ? nkx : 1;
            p.tap_off[e][t] = halo ? (kx == 0 ? 1 : 0) : 0;
            p.tap_w[e][t] = ky * 3 + kx;
        }
    }
    p.out_rs = 2;
    p.out_rb = a;
    p.out_cs = 2;
    p.out_cb = b;
    p.Hout = Hout;
    p.Wout = Wout;
    return p;
}

template <int BN>
size_t gemm_smem() {
    return 1024 + (size_t)gemm_stages<BN>() * (BM * BK * 2 + BN * BK * 2) + 8 * (2 * gemm_stages<BN>() + 5) + 16;
}

int sm_count() {
    static int sms[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!sms[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        sms[dev] = v > 0 ? v : 148;
    }
    return sms[dev];
}

template <int BN, int MODE = kModePlain>
int gemm_launch(const CUtensorMap& ma, const CUtensorMap& mb, void* C, int M, int N, int K, int ldc, const float* bias,
                int flags, int* err, int splits, int kt_per, int64_t split_stride, cudaStream_t s,
                ConvGeom cg = ConvGeom{1, 1, 1, 1, 1}) {
    // the shared-memory limit is a per-device attribute of the kernel: set
    // once per device
    static bool attr[64] = {false};
    int dev = 0;
    KGB_CUDA_TRY(cudaGetDevice(&dev));
    const size_t smem = gemm_smem<BN>();
    if (dev < 0 || dev >= 64 || !attr[dev]) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(gemm_tn_kernel<BN, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        if (dev >= 0 && dev < 64) attr[dev] = true;
    }
    const int tiles_m = (M + BM - 1) / BM, tiles_n = (N + BN - 1) / BN;
    const int64_t ntiles = (int64_t)tiles_m * tiles_n * splits;
    if (ntiles > 0x7fffffff) return set_error(KGB_ERR_VALUE, "gemm: too many tiles");
    // one persistent CTA per SM (at most one per tile)
    const int grid = (int)std::min<int64_t>(ntiles, sm_count());
    gemm_tn_kernel<BN, MODE><<<grid, kGemmThreads, smem, s>>>(ma, mb, C, M, N, K, ldc, bias, flags, err, kt_per,
                                                              split_stride, cg, tiles_m, tiles_n, splits);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

// C[m][n] = sum over z of work[z][m][n], in order z = 0, 1, ...
__global__ void splitk_sum_kernel(const float* __restrict__ work, float* __restrict__ C, int M, int N, int ldc,
                                  int splits) {
    const int64_t total = (int64_t)M * N;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int z = 0; z < splits; ++z) acc += work[z * total + i];
        C[(i / N) * ldc + (i % N)] = acc;
    }
}

int check_args(const void* A, const void* B, const void* C, int M, int N, int K, int lda, int ldb, int ldc) {
    if (!A || !B || !C) return set_error(KGB_ERR_VALUE, "gemm: null pointer");
    if (M <= 0 || N <= 0 || K <= 0) return set_error(KGB_ERR_VALUE, "gemm: sizes must be positive");
    if (K % 8 || lda % 8 || ldb % 8 || lda < K || ldb < K)
        return set_error(KGB_ERR_VALUE, "gemm: K and the leading dimensions must be multiples of 8 (16-byte rows)");
    if (((uintptr_t)A | (uintptr_t)B) & 15) return set_error(KGB_ERR_VALUE, "gemm: A and B must be 16-byte aligned");
    if (ldc < N) return set_error(KGB_ERR_VALUE, "gemm: ldc < N");
    return KGB_OK;
}

// 16-byte vector stores in the epilogue when every row segment is aligned
int vector_flag(const void* C, int ldc, int flags) {
    const int elems = (flags & 2) ? 8 : 4;
    return (((uintptr_t)C & 15) == 0 && ldc % elems == 0) ? 4 : 0;
}

int run_gemm(const void* A, const void* B, void* C, int M, int N, int K, int lda, int ldb, int ldc, const float* bias,
             int flags, int* err, int splits, int kt_per, int64_t split_stride, cudaStream_t s) {
    const int BN = N <= 64 ? 64 : 128;
    CUtensorMap ma, mb;
    int rc;
    if ((rc = make_map(&ma, A, M, K, lda, BM))) return rc;
    if ((rc = make_map(&mb, B, N, K, ldb, BN))) return rc;
    flags = (flags & 3) | vector_flag(C, ldc, flags);
    if (BN == 64) return gemm_launch<64>(ma, mb, C, M, N, K, ldc, bias, flags, err, splits, kt_per, split_stride, s);
    return gemm_launch<128>(ma, mb, C, M, N, K, ldc, bias, flags, err, splits, kt_per, split_stride, s);
}

}  // namespace
}  // namespace kgb

using namespace kgb;

extern "C" int kgb_gemm_bf16_tn(const void* A, const void* B, void* C, int M, int N, int K, int lda, int ldb, int ldc,
                                const float* bias, int flags, int* err_dev, void* stream) {
    int rc = check_args(A, B, C, M, N, K, lda, ldb, ldc);
    if (rc) return rc;
    const int ktiles = (K + BK - 1) / BK;
    return run_gemm(A, B, C, M, N, K, lda, ldb, ldc, bias, flags, err_dev, 1, ktiles, 0, (cudaStream_t)stream);
}

extern "C" int kgb_gemm_bf16_tn_splitk(const void* A, const void* B, float* C, int M, int N, int K, int lda, int ldb,
                                       int ldc, int splits, float* work, int64_t work_elems, int* err_dev,
                                       void* stream) {
    int rc = check_args(A, B, C, M, N, K, lda, ldb, ldc);
    if (rc) return rc;
    const int ktiles = (K + BK - 1) / BK;
    const int BN = N <= 64 ? 64 : 128;
    const int64_t tiles = (int64_t)((M + BM - 1) / BM) * ((N + BN - 1) / BN);
    if (splits <= 0) splits = (int)std::max<int64_t>(1, (2 * sm_count() + tiles - 1) / tiles);
    const int64_t mn = (int64_t)M * N;
    if (work && ((uintptr_t)work & 15) == 0) splits = (int)std::min<int64_t>(splits, work_elems / mn);
    else splits = 1;
    splits = std::max(1, std::min(splits, ktiles));
    // every split gets at least one k-tile
    const int kt_per = (ktiles + splits - 1) / splits;
    splits = (ktiles + kt_per - 1) / kt_per;
    cudaStream_t s = (cudaStream_t)stream;
    if (splits == 1) return run_gemm(A, B, C, M, N, K, lda, ldb, ldc, nullptr, 0, err_dev, 1, ktiles, 0, s);
    if ((rc = run_gemm(A, B, work, M, N, K, lda, ldb, N, nullptr, 0, err_dev, splits, kt_per, mn, s))) return rc;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((mn + 255) / 256, 4 * sm_count()));
    splitk_sum_kernel<<<grid, 256, 0, s>>>(work, C, M, N, ldc, splits);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

extern "C" int kgb_conv3x3_bf16(const void* x, const void* w, void* y, int B, int H, int W, int C, int N, int flip,
                                const float* bias, int flags, int* err_dev, void* stream) {
    if (!x || !w || !y) return set_error(KGB_ERR_VALUE, "conv: null pointer");
    if (B <= 0 || H <= 0 || W <= 0 || C <= 0 || N <= 0) return set_error(KGB_ERR_VALUE, "conv: sizes must be positive");
    if (C % 8) return set_error(KGB_ERR_VALUE, "conv: channels must be a multiple of 8 (16-byte pixel rows)");
    if (((uintptr_t)x | (uintptr_t)w) & 15) return set_error(KGB_ERR_VALUE, "conv: x and w must be 16-byte aligned");
    // 128-pixel M tiles as boxes of whole rows (W <= 128) or row segments (W >= 128)
    int bw, bh;
    if (W >= BM) {
        if (W % BM) return set_error(KGB_ERR_VALUE, "conv: width %d is neither a divisor nor a multiple of 128", W);
        bw = BM;
        bh = 1;
    } else {
        if (BM % W || H % (BM / W))
            return set_error(KGB_ERR_VALUE, "conv: %d x %d image does not tile into 128-pixel boxes", H, W);
        bw = W;
        bh = BM / W;
    }
    const int cblk = (C + BK - 1) / BK;
    const int K = 9 * cblk * BK;
    const int64_t M = (int64_t)B * H * W;
    if (M > 0x7fffffffLL) return set_error(KGB_ERR_VALUE, "conv: too many pixels");
    // N > 128: 256-column tiles, so each input box serves twice the columns
    // (the boxes per k-tile, not the MMAs, bound these small-image layers)
    const int BN = N <= 64 ? 64 : N <= 128 ? 128 : 256;
    CUtensorMap ma, mb;
    int rc;
    // rows of whole 128-pixel segments, one N tile, weights resident: read
    // each input row once per tile (conv_halo_kernel)
    const int hstages = W % BM == 0 && N <= 128 ? halo_stages(BN, cblk) : 0;
    if (hstages) {
        if ((rc = make_map_halo(&ma, x, B, H, W, C))) return rc;
        if ((rc = make_map(&mb, w, N, K, K, BN))) return rc;
        flags = (flags & 3) | vector_flag(y, N, flags);
        const ConvGeom hg{H, W, cblk, flip ? -1 : 1, B};
        const HaloPlan plan = plan_conv3x3(flip ? -1 : 1, H, W, C);
        cudaStream_t hs = (cudaStream_t)stream;
        if (BN == 64) return halo_launch<64>(ma, mb, y, (int)M, N, bias, flags, err_dev, hg, plan, hstages, hs);
        return halo_launch<128>(ma, mb, y, (int)M, N, bias, flags, err_dev, hg, plan, hstages, hs);
    }
    if ((rc = make_map_nhwc(&ma, x, B, H, W, C, bw, bh))) return rc;
    if ((rc = make_map(&mb, w, N, K, K, BN))) return rc;
    flags = (flags & 3) | vector_flag(y, N, flags);
    const ConvGeom cg{H, W, cblk, flip ? -1 : 1, B};
    cudaStream_t s = (cudaStream_t)stream;
    const int ktiles = K / BK;
    if (BN == 64)
        return gemm_launch<64, kModeConv>(ma, mb, y, (int)M, N, K, N, bias, flags, err_dev, 1, ktiles, 0, s, cg);
    if (BN == 128)
        return gemm_launch<128, kModeConv>(ma, mb, y, (int)M, N, K, N, bias, flags, err_dev, 1, ktiles, 0, s, cg);
    return gemm_launch<256, kModeConv>(ma, mb, y, (int)M, N, K, N, bias, flags, err_dev, 1, ktiles, 0, s, cg);
}

extern "C" int kgb_conv3x3_wgrad_bf16(const void* xT3, const void* gTr, float* dW, int B, int H, int W, int C, int N,
                                      int ldw, float* work, int64_t work_elems, int* err_dev, void* stream) {
    if (!xT3 || !gTr || !dW || !work) return set_error(KGB_ERR_VALUE, "wgrad: null pointer");
    if (B <= 0 || H <= 0 || W <= 0 || C <= 0 || N <= 0) return set_error(KGB_ERR_VALUE, "wgrad: sizes must be positive");
    if (C % 32) return set_error(KGB_ERR_VALUE, "wgrad: channels must be a multiple of 32");
    if (W % BK) return set_error(KGB_ERR_VALUE, "wgrad: width %d is not a multiple of %d", W, BK);
    if (ldw < 9 * C) return set_error(KGB_ERR_VALUE, "wgrad: ldw < 9 C");
    if ((((uintptr_t)xT3 | (uintptr_t)gTr | (uintptr_t)work) & 15) != 0)
        return set_error(KGB_ERR_VALUE, "wgrad: operands must be 16-byte aligned");
    const int64_t P = (int64_t)B * H * W;
    if (P > 0x7fffffffLL || (int64_t)3 * B > 0x7fffffffLL) return set_error(KGB_ERR_VALUE, "wgrad: too many pixels");
    // rows of A: per ky, the 3 C rows (kx, c) of the shifted copies, in
    // 128-row tiles (the last one zero-filled past 3 C)
    const int mt_ky = (3 * C + BM - 1) / BM;
    const int Mky = mt_ky * BM;
    const int M = 3 * Mky;
    const int BN = N <= 64 ? 64 : 128;
    const int64_t tiles = (int64_t)(M / BM) * ((N + BN - 1) / BN);
    const int ktiles = (int)(P / BK);
    const int64_t mn = (int64_t)M * N;
    if (work_elems < mn) return set_error(KGB_ERR_VALUE, "wgrad: work buffer smaller than the padded 9 C x N");
    // at most two tiles per SM: the persistent grid then ends evenly
    int splits = (int)std::max<int64_t>(1, (2 * sm_count()) / tiles);
    splits = (int)std::min<int64_t>(splits, work_elems / mn);
    splits = std::max(1, std::min(splits, ktiles));
    const int kt_per = (ktiles + splits - 1) / splits;
    splits = (ktiles + kt_per - 1) / kt_per;
    CUtensorMap ma, mb;
    int rc;
    if ((rc = make_map_wgrad(&ma, xT3, B, H, W, C))) return rc;
    if ((rc = make_map_rows(&mb, gTr, (int64_t)B * H, W, N, BN))) return rc;
    const ConvGeom cg{H, W, mt_ky, 1, B};
    cudaStream_t s = (cudaStream_t)stream;
    const int flags = vector_flag(work, N, 0);
    if (BN == 64) rc = gemm_launch<64, kModeWgrad>(ma, mb, work, M, N, (int)P, N, nullptr, flags, err_dev, splits, kt_per,
                                                   mn, s, cg);
    else rc = gemm_launch<128, kModeWgrad>(ma, mb, work, M, N, (int)P, N, nullptr, flags, err_dev, splits, kt_per, mn,
                                           s, cg);
    if (rc) return rc;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((mn + 255) / 256, 4 * sm_count()));
    wgrad_sum_kernel<<<grid, 256, 0, s>>>(work, dW, M, N, splits, C, Mky, ldw);
    KGB_CUDA_TRY(cudaGetLastError());
    return KGB_OK;
}

extern "C" int kgb_conv3x3_s2_dgrad_bf16(const void* g, const void* wt, float* dx, int B, int Hg, int Wg, int C, int N,
                                        int* err_dev, void* stream) {
    if (!g || !wt || !dx) return set_error(KGB_ERR_VALUE, "s2 dgrad: null pointer");
    if (B <= 0 || Hg <= 0 || Wg <= 0 || C <= 0 || N <= 0) return set_error(KGB_ERR_VALUE, "s2 dgrad: sizes must be positive");
    if (C % 8) return set_error(KGB_ERR_VALUE, "s2 dgrad: channels must be a multiple of 8 (16-byte pixel rows)");
    const bool halo = Wg % BM == 0;
    const bool rows = !halo && Wg % 32 == 0 && BM % Wg == 0 && Hg % (BM / Wg) == 0;
    if (!(halo || rows) || N > 128 || N % 4)
        return set_error(KGB_ERR_VALUE,
                         "s2 dgrad: needs gradient rows of 128-pixel multiples (or of 32 or 64 pixels with whole "
                         "128-pixel tiles per image) and N <= 128, N %% 4 == 0");
    if ((((uintptr_t)g | (uintptr_t)wt | (uintptr_t)dx) & 15) != 0)
        return set_error(KGB_ERR_VALUE, "s2 dgrad: operands must be 16-byte aligned");
    const int cblk = (C + BK - 1) / BK;
    const int K = 9 * cblk * BK;
    const int64_t M = (int64_t)B * Hg * Wg;
    if (M > 0x7fffffffLL) return set_error(KGB_ERR_VALUE, "s2 dgrad: too many pixels");
    const int BN = N <= 64 ? 64 : 128;
    const int hstages = halo_stages(BN, cblk);
    if (!hstages) return set_error(KGB_ERR_NOT_IMPLEMENTED, "s2 dgrad: weights do not fit in shared memory");
    CUtensorMap ma, mb;
    int rc;
    if ((rc = halo ? make_map_halo(&ma, g, B, Hg, Wg, C) : make_map_nhwc(&ma, g, B, Hg, Wg, C, Wg, BM / Wg))) return rc;
    if ((rc = make_map(&mb, wt, N, K, K, BN))) return rc;
    const int flags = vector_flag(dx, 2 * N, 0);
    const ConvGeom hg{Hg, Wg, cblk, 1, B};
    cudaStream_t s = (cudaStream_t)stream;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            const HaloPlan plan = plan_s2_dgrad(a, b, 2 * Hg, 2 * Wg, C, halo);
            rc = BN == 64 ? halo_launch<64>(ma, mb, dx, (int)M, N, nullptr, flags, err_dev, hg, plan, hstages, s)
                          : halo_launch<128>(ma, mb, dx, (int)M, N, nullptr, flags, err_dev, hg, plan, hstages, s);
            if (rc) return rc;
        }
    return KGB_OK;
}
