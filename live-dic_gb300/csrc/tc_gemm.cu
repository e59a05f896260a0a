// BF16 tensor-core GEMM for the learned seed network (sm_103a, tcgen05).
//
//   D[m, n] (+)= sum_k A[m, k] * B[n, k]   (+ bias[n], ReLU)
//
// A (M x K) and B (N x K) are row-major BF16 with K contiguous ("K-major");
// D is FP32 and/or BF16 with row stride ldd.  M is a multiple of 128, N of
// the tile width BN, K (per split) of 64; callers pad.
//
// One CTA per 128 x BN output tile (x one K split), 128 threads:
//   * thread 0 of warp 0 issues TMA loads of 128x64 A and BNx64 B tiles
//     (128-byte swizzle) into a 4-stage shared-memory ring, each stage
//     guarded by a full/empty mbarrier pair;
//   * thread 0 of warp 1 issues tcgen05.mma (M=128, N=BN, K=16, FP32
//     accumulator in tensor memory), four per 64-wide stage, and releases
//     each stage with tcgen05.commit on its empty barrier;
//   * after the last commit all four warps read their 32 accumulator lanes
//     with tcgen05.ld and apply the epilogue.
// Convolution GEMMs can gather operand A in the kernel (implicit GEMM):
// warps 2 and 3 then fill each stage's A tile with 16-byte cp.async copies
// straight from the NHWC tensor (an im2col row of the forward, or the
// data-gradient gather of the output gradient; zero-filled outside the
// image), at the positions the 128-byte swizzle gives them, and each warp
// arrives on the stage's full barrier after its copies landed and were
// fenced to the async proxy that tcgen05.mma reads through; TMA still
// loads B.  The 9x-expanded im2col matrix is never written or read.
// Every mbarrier wait is bounded: on expiry the CTA records an error code and
// carries on, so a fault of the pipeline ends the kernel instead of hanging.
// Before a failed CTA frees its tensor memory and exits, it waits (bounded
// again) for the copies of every stage the producer armed but the MMA issuer
// never consumed, and for the MMAs it did issue, so no bulk copy or MMA is
// left writing into the CTA's shared or tensor memory.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>

#include "gbdic_kernels.h"

namespace gbdic {
namespace {

constexpr int kStages = 4;
constexpr int kBM = 128;
constexpr int kBK = 64;
constexpr uint32_t kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded parity wait; returns false on expiry.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t addr = smem_u32(bar);
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// 16 bytes from global to shared memory; src_bytes 0 writes zeros.
__device__ __forceinline__ void cp_async_16(uint32_t dst, const void *src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}

// Chunk q (K elements 8q .. 8q+7) of row m of the gathered operand, or
// nullptr where it is zero.  Same mapping as im2col_vec_kernel /
// dgrad_gather_vec_kernel (nn_ops.cu): C (Cout) % 8 == 0, so a chunk never
// straddles two taps.
__device__ __forceinline__ const uint4 *gather_chunk(const TcGemmArgs &a, int m, int q) {
    const NnConvShape &s = a.conv;
    const uint4 *src = static_cast<const uint4 *>(a.a);
    const int k0 = 8 * q;
    if (a.gather == kGatherIm2col) {
        if (k0 >= 9 * s.C) return nullptr;
        const int tap = k0 / s.C, ci0 = k0 - tap * s.C, ky = tap / 3, kx = tap - 3 * ky;
        const int ox = m % s.OW, t = m / s.OW, oy = t % s.OH, b = t / s.OH;
        const int iy = 2 * oy + ky - 1, ix = 2 * ox + kx - 1;
        if (iy < 0 || iy >= s.H || ix < 0 || ix >= s.W) return nullptr;
        return src + ((((size_t)b * s.H + iy) * s.W + ix) * s.C + ci0) / 8;
    }
    const int tap = k0 / s.Cout, co0 = k0 - tap * s.Cout, ky = tap / 3, kx = tap - 3 * ky;
    const int ix = m % s.W, t = m / s.W, iy = t % s.H, b = t / s.H;
    const int ty = iy + 1 - ky, tx = ix + 1 - kx;
    if (ty < 0 || tx < 0 || (ty & 1) || (tx & 1) || (ty >> 1) >= s.OH || (tx >> 1) >= s.OW) return nullptr;
    return src + ((((size_t)b * s.OH + (ty >> 1)) * s.OW + (tx >> 1)) * s.Cout + co0) / 8;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), leading offset unused for swizzled K-major (1).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;                  // LBO (unused)
    d |= (uint64_t)(1024u >> 4) << 32;        // SBO
    d |= (uint64_t)1u << 46;                  // descriptor version (sm_100 family)
    d |= (uint64_t)2u << 61;                  // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <int BN>
__global__ void __launch_bounds__(128, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap map_a,
                                                         const __grid_constant__ CUtensorMap map_b,
                                                         TcGemmArgs args) {
    constexpr uint32_t kBytesA = kBM * kBK * 2;
    constexpr uint32_t kBytesB = BN * kBK * 2;
    constexpr uint32_t kStageBytes = kBytesA + kBytesB;
    constexpr uint32_t kTmemCols = BN < 32 ? 32 : BN;
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t full_bar[kStages], empty_bar[kStages], done_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int failed;
    __shared__ int issued_kb, consumed_kb;  // K blocks whose loads were issued / consumed

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int n0 = blockIdx.x * BN, m0 = blockIdx.y * kBM;
    const int k_len = args.K / args.k_split;
    const int k_begin = blockIdx.z * k_len;
    const int num_kb = k_len / kBK;

    if (tid == 0) {
        // Full barriers: the TMA producer's arrive (with the stage's bytes),
        // plus one arrive per gathering warp in gather mode.
        const uint32_t full_count = args.gather ? 3u : 1u;
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full_bar[s], full_count);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&done_bar, 1);
        failed = 0;
        issued_kb = 0;
        consumed_kb = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTmemCols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    if (warp == 0 && lane == 0) {
        // TMA producer.
        int kb = 0;
        for (; kb < num_kb; ++kb) {
            const int s = kb % kStages;
            if (kb >= kStages && !mbar_wait(&empty_bar[s], ((kb / kStages) - 1) & 1)) {
                atomicExch(&failed, 1);
                break;
            }
            uint8_t *sa = smem + s * kStageBytes;
            uint8_t *sb = sa + kBytesA;
            mbar_expect_tx(&full_bar[s], args.gather ? kBytesB : kStageBytes);
            const int kx = k_begin + kb * kBK;
            if (!args.gather) tma_load_2d(sa, &map_a, &full_bar[s], kx, m0);
            tma_load_2d(sb, &map_b, &full_bar[s], kx, n0);
        }
        issued_kb = kb;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer.
        constexpr uint32_t idesc = instr_desc(kBM, BN);
        int kb = 0;
        for (; kb < num_kb; ++kb) {
            const int s = kb % kStages;
            if (!mbar_wait(&full_bar[s], (kb / kStages) & 1)) {
                atomicExch(&failed, 1);
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_addr = smem_u32(smem + s * kStageBytes);
            const uint32_t b_addr = a_addr + kBytesA;
#pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk) {
                const uint64_t da = smem_desc(a_addr + kk * 32);
                const uint64_t db = smem_desc(b_addr + kk * 32);
                const uint32_t accumulate = (kb > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(accumulate));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&empty_bar[s]))
                         : "memory");
        }
        consumed_kb = kb;
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&done_bar))
                     : "memory");
    }
    if (args.gather && warp >= 2) {
        // Operand A producers: 64 threads, thread g copies chunk g % 8 of
        // rows g / 8 + 8 i (i < 16) of the 128 x 64 tile, so eight threads
        // read one row's 128 contiguous bytes.  Row r, chunk j lands at byte
        // r * 128 + ((j ^ (r % 8)) * 16) of the 1024-byte-aligned stage, the
        // 128-byte swizzle of the TMA loads it replaces.
        const int g = tid - 64, j = g & 7;
        for (int kb = 0; kb < num_kb; ++kb) {
            const int s = kb % kStages;
            if (kb >= kStages) {
                int ok = 1;
                if (lane == 0) ok = mbar_wait(&empty_bar[s], ((kb / kStages) - 1) & 1) ? 1 : 0;
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) atomicExch(&failed, 1);
                    break;
                }
            }
            const uint32_t sa = smem_u32(smem + s * kStageBytes);
            const int q = (k_begin + kb * kBK) / 8 + j;
#pragma unroll 4
            for (int i = 0; i < 16; ++i) {
                const int r = (g >> 3) + 8 * i;
                const uint4 *src = gather_chunk(args, m0 + r, q);
                cp_async_16(sa + (uint32_t)(r * 128 + ((j ^ (r & 7)) << 4)), src ? src : args.a, src ? 16u : 0u);
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&full_bar[s]);
        }
    }
    __syncwarp();
    if (!mbar_wait(&done_bar, 0)) atomicExch(&failed, 1);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // Epilogue: warp w owns accumulator lanes (rows) 32w .. 32w + 31.
    const int row = m0 + warp * 32 + lane;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
        uint32_t r[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
            "%14, %15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(tmem + lane_base + (uint32_t)c));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            v[j] = __uint_as_float(r[j]);
            if (args.bias) v[j] = v[j] + args.bias[n0 + c + j];
            if (args.relu) v[j] = fmaxf(v[j], 0.0f);
        }
        const size_t base = (size_t)blockIdx.z * (size_t)args.split_stride + (size_t)row * args.ldd + n0 + c;
        if (args.d_f32) {
            float4 *o = reinterpret_cast<float4 *>(args.d_f32 + base);
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                float4 x = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
                if (args.accumulate) {
                    const float4 y = o[j];
                    x.x += y.x; x.y += y.y; x.z += y.z; x.w += y.w;
                }
                o[j] = x;
            }
        }
        if (args.d_bf16) {
            __nv_bfloat162 *o = reinterpret_cast<__nv_bfloat162 *>(static_cast<__nv_bfloat16 *>(args.d_bf16) + base);
#pragma unroll
            for (int j = 0; j < 8; ++j) o[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        if (lane == 0 && failed) {
            // The producer runs at most kStages K blocks ahead of the issuer,
            // so the unconsumed blocks occupy distinct stages.
            for (int kb = consumed_kb; kb < issued_kb; ++kb) mbar_wait(&full_bar[kb % kStages], (kb / kStages) & 1);
            mbar_wait(&done_bar, 0);
        }
        __syncwarp();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
    }
    if (tid == 0 && failed && args.error) atomicExch(args.error, 1);
}

typedef CUresult (*EncodeTiled)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

// 2-D BF16 row-major matrix rows x cols (cols contiguous), box box_rows x 64.
bool make_map(CUtensorMap *map, const void *ptr, int rows, int cols, int box_rows) {
    EncodeTiled fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    const cuuint32_t estride[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estride,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
cudaError_t launch_bn(const CUtensorMap &ma, const CUtensorMap &mb, const TcGemmArgs &a, cudaStream_t stream) {
    const size_t smem = (size_t)kStages * (kBM * kBK * 2 + BN * kBK * 2) + 1024;
    // The attribute is per device; set it once per device and tile width.
    static thread_local int configured_device = -1;
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return err;
    if (configured_device != device) {
        err = cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (err != cudaSuccess) return err;
        configured_device = device;
    }
    dim3 grid(a.N / BN, a.M / kBM, a.k_split);
    tc_gemm_kernel<BN><<<grid, 128, smem, stream>>>(ma, mb, a);
    return cudaGetLastError();
}

}  // namespace

int tc_gemm_tile_n(int N) {
    if (N % 128 == 0) return 128;
    if (N % 64 == 0) return 64;
    if (N % 32 == 0) return 32;
    if (N % 16 == 0) return 16;
    return 0;
}

cudaError_t launch_tc_gemm(const TcGemmArgs &a, cudaStream_t stream) {
    const int bn = tc_gemm_tile_n(a.N);
    if (a.M <= 0 || a.N <= 0 || a.K <= 0 || a.k_split < 1 || a.M % kBM != 0 || bn == 0 ||
        a.K % (kBK * a.k_split) != 0 || a.ldd < a.N || a.ldd % 4 != 0 || !a.a || !a.b ||
        (!a.d_f32 && !a.d_bf16) || (a.accumulate && !a.d_f32) || (a.k_split > 1 && a.bias))
        return cudaErrorInvalidValue;
    if ((reinterpret_cast<uintptr_t>(a.a) | reinterpret_cast<uintptr_t>(a.b)) & 15u) return cudaErrorMisalignedAddress;
    if (a.gather != kGatherNone) {
        // The gathered operand's rows and reduction length must be the
        // convolution's exactly (every row and chunk maps into the tensor).
        const NnConvShape &s = a.conv;
        if (a.k_split != 1 || s.B < 1 || s.H < 1 || s.W < 1 || s.OH != (s.H + 1) / 2 || s.OW != (s.W + 1) / 2)
            return cudaErrorInvalidValue;
        if (a.gather == kGatherIm2col) {
            if (s.C < 8 || s.C % 8 || a.M != s.B * s.OH * s.OW || a.K != s.Kp || s.Kp < 9 * s.C)
                return cudaErrorInvalidValue;
        } else if (a.gather == kGatherDgrad) {
            if (s.Cout < 8 || s.Cout % 8 || a.M != s.B * s.H * s.W || a.K != 9 * s.Cout) return cudaErrorInvalidValue;
        } else {
            return cudaErrorInvalidValue;
        }
    }
    CUtensorMap ma, mb;
    if (!make_map(&mb, a.b, a.N, a.K, bn)) return cudaErrorInvalidValue;
    if (a.gather == kGatherNone) {
        if (!make_map(&ma, a.a, a.M, a.K, kBM)) return cudaErrorInvalidValue;
    } else {
        ma = mb;  // not read: operand A is gathered
    }
    switch (bn) {
    case 128: return launch_bn<128>(ma, mb, a, stream);
    case 64: return launch_bn<64>(ma, mb, a, stream);
    case 32: return launch_bn<32>(ma, mb, a, stream);
    default: return launch_bn<16>(ma, mb, a, stream);
    }
}

}  // namespace gbdic
