// BF16 "TN" GEMM on the 5th-generation tensor cores (tcgen05) for sm_103a:
//   C[m][n] = sum_k A[m][k] * B[n][k]  (+ bias[n], optional ReLU)
// A (M x K) and B (N x K) are row-major bf16 with K contiguous; C is float32
// or bf16 with leading dimension ldc.  This is the one tensor-core kernel of
// the U-Net preconditioner: its convolutions (forward, data gradient, weight
// gradient) are lowered to it through im2col / transposes.
//
// Structure (one 128 x BN output tile per CTA, 4 warps):
//  * warp 0, one lane: TMA producer -- 2-D tiled bulk-tensor loads of the A
//    and B k-tiles (64 bf16 = 128 bytes along K) with 128-byte swizzle into a
//    STAGES-deep shared-memory ring, completion counted on "full" mbarriers;
//  * warp 1, one lane: MMA issuer -- four tcgen05.mma (K = 16 each) per
//    k-tile on shared-memory descriptors, accumulating in tensor memory;
//    tcgen05.commit releases the stage ("empty" mbarrier) and finally signals
//    the epilogue;
//  * warp 2 allocates and frees the tensor-memory accumulator (BN columns);
//  * all four warps run the epilogue: tcgen05.ld of their 32 accumulator
//    lanes, bias / ReLU, store.
// Every mbarrier wait is bounded: after ~2^26 polls the CTA records an error
// code in `err` and leaves (tensor memory is still freed).
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "kgb_internal.h"

namespace kgb {
namespace {

constexpr int BM = 128;
constexpr int BK = 64;          // bf16 elements per k-tile row = 128 bytes (one swizzle atom)
constexpr int STAGES = 4;
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
// convolution of the data gradient).
struct ConvGeom {
    int H, W, cblk, sgn;
};

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

template <int BN, bool CONV>
__global__ void __launch_bounds__(128, 1)
gemm_tn_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, void* __restrict__ C,
               int M, int N, int K, int ldc, const float* __restrict__ bias, int flags, int* __restrict__ err,
               int kt_per, int64_t split_stride, const ConvGeom cg) {
    constexpr int A_BYTES = BM * BK * 2;
    constexpr int B_BYTES = BN * BK * 2;
    extern __shared__ uint8_t smem_dyn[];
    // 1024-byte alignment for the swizzled tiles
    const uint32_t base_s = smem_u32(smem_dyn);
    const uint32_t pad = (1024 - (base_s & 1023)) & 1023;
    uint8_t* smem = smem_dyn + pad;
    const uint32_t sA = smem_u32(smem);
    const uint32_t sB = sA + STAGES * A_BYTES;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem + STAGES * (A_BYTES + B_BYTES));
    // bars[0..S) full, bars[S..2S) empty, bars[2S] done; then the tmem slot and an abort flag
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
    const uint32_t bar_full = smem_u32(bars);
    const uint32_t bar_empty = bar_full + 8 * STAGES;
    const uint32_t bar_done = bar_full + 16 * STAGES;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    // split-K: this CTA reduces k-tiles [kt0, kt0 + ktiles) into its own
    // slice of C (the host makes every slice non-empty)
    const int kt0 = blockIdx.z * kt_per;
    const int ktiles = min((K + BK - 1) / BK - kt0, kt_per);
    if (blockIdx.z) C = reinterpret_cast<float*>(C) + blockIdx.z * split_stride;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(bar_full + 8 * s, 1);
            mbar_init(bar_empty + 8 * s, 1);
        }
        mbar_init(bar_done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 2) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"((uint32_t)BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // producer
        int img = 0, h0 = 0, w0 = 0;
        if (CONV) {
            const int hw = cg.H * cg.W;
            img = m0 / hw;
            const int r = m0 - img * hw;
            h0 = r / cg.W;
            w0 = r - h0 * cg.W;
        }
        for (int kt = 0; kt < ktiles; ++kt) {
            const int s = kt % STAGES;
            if (kt >= STAGES && !mbar_wait(bar_empty + 8 * s, ((kt / STAGES) - 1) & 1)) {
                *abort_flag = 1;
                break;
            }
            mbar_expect_tx(bar_full + 8 * s, A_BYTES + B_BYTES);
            if (CONV) {
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
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = idesc_bf16(BM, BN);
        bool ok = true;
        for (int kt = 0; kt < ktiles; ++kt) {
            const int s = kt % STAGES;
            if (!mbar_wait(bar_full + 8 * s, (kt / STAGES) & 1)) {
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
                    ::"r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(acc));
            }
            // release the stage when these MMAs have read it
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(bar_empty + 8 * s) : "memory");
        }
        if (!ok) *abort_flag = 1;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     ::"r"(bar_done) : "memory");
    }
    __syncwarp();
    // epilogue: every warp reads its 32 accumulator lanes
    const bool done = mbar_wait(bar_done, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const bool good = done && !*abort_flag;
    const int row = m0 + warp * 32 + lane;
    for (int c0 = 0; c0 < BN; c0 += 32) {
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
            "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
              "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (good && row < M && (flags & 4) && n0 + c0 + 32 <= N) {
            // whole 32-column chunk, 16-byte aligned row segment
            float v[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                v[j] = __uint_as_float(r[j]);
                if (bias) v[j] += __ldg(bias + n0 + c0 + j);
                if (flags & 1) v[j] = fmaxf(v[j], 0.f);
            }
            if (flags & 2) {
                uint4* dst = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(C) + (size_t)row * ldc + n0 + c0);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    uint4 u;
                    u.x = pack_bf16(v[8 * q + 0], v[8 * q + 1]);
                    u.y = pack_bf16(v[8 * q + 2], v[8 * q + 3]);
                    u.z = pack_bf16(v[8 * q + 4], v[8 * q + 5]);
                    u.w = pack_bf16(v[8 * q + 6], v[8 * q + 7]);
                    dst[q] = u;
                }
            } else {
                float4* dst = reinterpret_cast<float4*>(reinterpret_cast<float*>(C) + (size_t)row * ldc + n0 + c0);
#pragma unroll
                for (int q = 0; q < 8; ++q) dst[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        } else if (good && row < M) {
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int col = n0 + c0 + j;
                if (col < N) {
                    float v = __uint_as_float(r[j]);
                    if (bias) v += __ldg(bias + col);
                    if (flags & 1) v = fmaxf(v, 0.f);
                    if (flags & 2)
                        reinterpret_cast<__nv_bfloat16*>(C)[(size_t)row * ldc + col] = __float2bfloat16(v);
                    else
                        reinterpret_cast<float*>(C)[(size_t)row * ldc + col] = v;
                }
            }
        }
    }
    if (!good && threadIdx.x == 0 && err) atomicExch(err, 1);
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 2) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((uint32_t)BN));
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

template <int BN>
size_t gemm_smem() {
    return 1024 + (size_t)STAGES * (BM * BK * 2 + BN * BK * 2) + 8 * (2 * STAGES + 1) + 16;
}

template <int BN, bool CONV = false>
int gemm_launch(const CUtensorMap& ma, const CUtensorMap& mb, void* C, int M, int N, int K, int ldc, const float* bias,
                int flags, int* err, int splits, int kt_per, int64_t split_stride, cudaStream_t s,
                ConvGeom cg = ConvGeom{1, 1, 1, 1}) {
    static bool attr = false;
    const size_t smem = gemm_smem<BN>();
    if (!attr) {
        KGB_CUDA_TRY(cudaFuncSetAttribute(gemm_tn_kernel<BN, CONV>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        attr = true;
    }
    dim3 grid((unsigned)((M + BM - 1) / BM), (unsigned)((N + BN - 1) / BN), (unsigned)splits);
    gemm_tn_kernel<BN, CONV><<<grid, 128, smem, s>>>(ma, mb, C, M, N, K, ldc, bias, flags, err, kt_per, split_stride,
                                                     cg);
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
    if (splits <= 0) splits = (int)std::max<int64_t>(1, (2 * 152 + tiles - 1) / tiles);
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
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((mn + 255) / 256, 4 * 152));
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
    const int BN = N <= 64 ? 64 : 128;
    CUtensorMap ma, mb;
    int rc;
    if ((rc = make_map_nhwc(&ma, x, B, H, W, C, bw, bh))) return rc;
    if ((rc = make_map(&mb, w, N, K, K, BN))) return rc;
    flags = (flags & 3) | vector_flag(y, N, flags);
    const ConvGeom cg{H, W, cblk, flip ? -1 : 1};
    cudaStream_t s = (cudaStream_t)stream;
    const int ktiles = K / BK;
    if (BN == 64)
        return gemm_launch<64, true>(ma, mb, y, (int)M, N, K, N, bias, flags, err_dev, 1, ktiles, 0, s, cg);
    return gemm_launch<128, true>(ma, mb, y, (int)M, N, K, N, bias, flags, err_dev, 1, ktiles, 0, s, cg);
}
