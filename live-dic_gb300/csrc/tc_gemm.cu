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
// the CTA then has 64 + 32 kGatherWarps threads, and warps 2 and up fill
// each stage's A tile with 16-byte cp.async copies
// straight from the NHWC tensor (an im2col row of the forward, or the
// data-gradient gather of the output gradient; zero-filled outside the
// image), at the positions the 128-byte swizzle gives them, from a table of
// the tile's 128 row origins built once per CTA; each warp arrives on a
// stage's full barrier once that stage's copies landed and were fenced to
// the async proxy that tcgen05.mma reads through, while its next stage's
// copies are in flight; TMA still loads B.  The 9x-expanded im2col matrix is never
// written or read.  The data-gradient GEMM orders its rows by the input
// pixel's stride-2 parity class and skips the K blocks of the taps that are
// zero for the tile's class (9 of the 36 class-tap pairs remain).  The
// ring has min(4, K blocks) stages (2 in gather mode, where the copies, not
// the ring, set the pace), so short K loops and gathering CTAs need little
// shared memory and more CTAs stay resident.
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

#ifndef GBDIC_GEMM_STAGES
#define GBDIC_GEMM_STAGES 4
#endif
#ifndef GBDIC_GATHER_AHEAD
#define GBDIC_GATHER_AHEAD 1
#endif
#ifndef GBDIC_GATHER_WARPS
#define GBDIC_GATHER_WARPS 8
#endif
#ifndef GBDIC_GATHER_STAGES
#define GBDIC_GATHER_STAGES 2
#endif
constexpr int kStages = GBDIC_GEMM_STAGES;
// Ring depth in gather mode (<= kStages): the gathers keep only a few
// stages in flight, so a shallower ring leaves room for more resident CTAs.
constexpr int kGatherStages = GBDIC_GATHER_STAGES;
static_assert(kGatherStages >= 2 && kGatherStages <= kStages, "gather ring depth");
// Gather mode: warps 2 .. 2 + kGatherWarps - 1 fill operand A.
constexpr int kGatherWarps = GBDIC_GATHER_WARPS;
constexpr int kGatherThreads = 32 * kGatherWarps;
constexpr int kMaxThreads = 64 + kGatherThreads;
static_assert(kGatherWarps == 2 || kGatherWarps == 4 || kGatherWarps == 8, "1024 chunks per stage split evenly");
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

// Row descriptor of the gathered operand, built once per CTA: the chunk
// (8-element) offset of the row's pixel origin in the NHWC source and the
// origin's coordinates.  im2col row m = (b, oy, ox): origin (2 oy - 1,
// 2 ox - 1) of input image b, tap (ky, kx) reads pixel (y + ky, x + kx).
// Data-gradient row m = (b, iy, ix): origin (iy + 1, ix + 1), tap (ky, kx)
// reads output-gradient pixel ((y - ky) / 2, (x - kx) / 2) when both are
// even and inside the OH x OW grid.  Same mapping as im2col_vec_kernel /
// dgrad_gather_vec_kernel (nn_ops.cu).
//
// Parity classes (kGatherDgradClasses, even H and W): the rows are ordered
// by class c = 2 py + px of the input pixel (iy, ix) = (2u + py, 2v + px),
// then by (b, u, v); a class holds B OH OW rows (a multiple of 128), so a
// tile never mixes classes.  In class (py, px) the tap (ky, kx) is nonzero
// only for ky = 1 (py = 0) or ky in {0, 2} (py = 1), likewise kx, and reads
// output-gradient pixel (u + dy, v + dx), dy = 1 for (py, ky) = (1, 0), else
// 0.  The other taps' K blocks are zero for every row of the tile and are
// skipped: they would add exact zeros to the accumulator.
__device__ __forceinline__ int4 gather_row(const TcGemmArgs &a, int m) {
    const NnConvShape &s = a.conv;
    if (a.gather == kGatherIm2col) {
        const int ox = m % s.OW, t = m / s.OW, oy = t % s.OH, b = t / s.OH;
        const int y = 2 * oy - 1, x = 2 * ox - 1;
        return make_int4(((b * s.H + y) * s.W + x) * (s.C / 8), y, x, 0);
    }
    if (a.gather == kGatherDgradClasses) {
        const int local = m % (s.B * s.OH * s.OW);
        const int v = local % s.OW, t = local / s.OW, u = t % s.OH, b = t / s.OH;
        return make_int4(((b * s.OH + u) * s.OW + v) * (s.Cout / 8), u, v, 0);
    }
    const int ix = m % s.W, t = m / s.W, iy = t % s.H, b = t / s.H;
    return make_int4(b * s.OH * s.OW * (s.Cout / 8), iy + 1, ix + 1, 0);
}

// Parity class of the tile starting at row m0 (class mode), else 0.
__device__ __forceinline__ int gather_class(const TcGemmArgs &a, int m0) {
    return a.gather == kGatherDgradClasses ? m0 / (a.conv.B * a.conv.OH * a.conv.OW) : 0;
}

// K blocks of one CTA: all of its split, or in class mode those of the
// class's nonzero taps (Cout / 64 blocks per tap).
__device__ __forceinline__ int kblock_count(const TcGemmArgs &a, int k_len, int cls) {
    if (a.gather != kGatherDgradClasses) return k_len / kBK;
    return ((cls >> 1) ? 2 : 1) * ((cls & 1) ? 2 : 1) * (a.conv.Cout / kBK);
}

// First K element of the CTA's kb-th K block.
__device__ __forceinline__ int kblock_offset(const TcGemmArgs &a, int kb, int k_begin, int cls) {
    if (a.gather != kGatherDgradClasses) return k_begin + kb * kBK;
    const int per_tap = a.conv.Cout / kBK, t = kb / per_tap, within = kb - t * per_tap;
    const int nx = (cls & 1) ? 2 : 1, ty = t / nx, tx = t - ty * nx;
    const int ky = (cls >> 1) ? 2 * ty : 1, kx = (cls & 1) ? 2 * tx : 1;
    return (ky * 3 + kx) * a.conv.Cout + within * kBK;
}

// Tap of the chunk starting at K element k0: C (Cout) % 8 == 0, so a chunk
// never straddles two taps.  im2col: (ky, kx, the tap's chunk offset, 0 for
// the K padding beyond 9 C); data gradient: (ky, kx, channel chunk, 1);
// class mode: (dy, dx, chunk offset of pixel (dy, dx) and channel, 1).
__device__ __forceinline__ int4 gather_tap(const TcGemmArgs &a, int k0, int cls) {
    const NnConvShape &s = a.conv;
    const int per_tap = (a.gather == kGatherIm2col ? s.C : s.Cout) / 8;
    const int q = k0 / 8, tap = q / per_tap, c8 = q - tap * per_tap, ky = tap / 3, kx = tap - 3 * ky;
    if (a.gather == kGatherIm2col) return make_int4(ky, kx, (ky * s.W + kx) * per_tap + c8, tap < 9 ? 1 : 0);
    if (a.gather == kGatherDgradClasses) {
        const int dy = ((cls >> 1) && ky == 0) ? 1 : 0, dx = ((cls & 1) && kx == 0) ? 1 : 0;
        return make_int4(dy, dx, (dy * s.OW + dx) * per_tap + c8, 1);
    }
    return make_int4(ky, kx, c8, 1);
}

// Source chunk of (row, tap), or nullptr where the operand is zero.
__device__ __forceinline__ const uint4 *gather_src(const TcGemmArgs &a, int4 row, int4 tap) {
    const NnConvShape &s = a.conv;
    const uint4 *src = static_cast<const uint4 *>(a.a);
    if (a.gather == kGatherIm2col) {
        const int yy = row.y + tap.x, xx = row.z + tap.y;
        if (!tap.w || (unsigned)yy >= (unsigned)s.H || (unsigned)xx >= (unsigned)s.W) return nullptr;
        return src + (row.x + tap.z);
    }
    if (a.gather == kGatherDgradClasses) {
        if (row.y + tap.x >= s.OH || row.z + tap.y >= s.OW) return nullptr;
        return src + (row.x + tap.z);
    }
    const int ty = row.y - tap.x, tx = row.z - tap.y;
    if (((ty | tx) & 1) || (unsigned)ty >= (unsigned)(2 * s.OH) || (unsigned)tx >= (unsigned)(2 * s.OW)) return nullptr;
    return src + (row.x + ((ty >> 1) * s.OW + (tx >> 1)) * (s.Cout / 8) + tap.z);
}

// Output row of accumulator row m (class mode: back to (b, iy, ix) order).
__device__ __forceinline__ int output_row(const TcGemmArgs &a, int m, int cls) {
    if (a.gather != kGatherDgradClasses) return m;
    const NnConvShape &s = a.conv;
    const int local = m - cls * (s.B * s.OH * s.OW);
    const int v = local % s.OW, t = local / s.OW, u = t % s.OH, b = t / s.OH;
    return (b * s.H + 2 * u + (cls >> 1)) * s.W + 2 * v + (cls & 1);
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
__global__ void __launch_bounds__(kMaxThreads, 1) tc_gemm_kernel(const __grid_constant__ CUtensorMap map_a,
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
    __shared__ int4 row_tab[kBM];           // gather mode: descriptors of the tile's rows

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *smem = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int n0 = blockIdx.x * BN, m0 = blockIdx.y * kBM;
    const int k_len = args.K / args.k_split;
    const int k_begin = blockIdx.z * k_len;
    const int cls = gather_class(args, m0);
    const int num_kb = kblock_count(args, k_len, cls);
    // The ring holds min(4, K blocks) stages (launch_bn sizes the dynamic
    // shared memory the same way), so short K loops leave room for more
    // resident CTAs.
    const int ring = args.gather ? kGatherStages : kStages;
    const int nst = num_kb < ring ? num_kb : ring;

    if (args.gather && tid < kBM) row_tab[tid] = gather_row(args, m0 + tid);
    if (tid == 0) {
        // Full barriers: the TMA producer's arrive (with the stage's bytes),
        // plus one arrive per gathering warp in gather mode.
        const uint32_t full_count = args.gather ? 1u + (uint32_t)kGatherWarps : 1u;
        for (int s = 0; s < nst; ++s) {
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
            const int s = kb % nst;
            if (kb >= nst && !mbar_wait(&empty_bar[s], ((kb / nst) - 1) & 1)) {
                atomicExch(&failed, 1);
                break;
            }
            uint8_t *sa = smem + s * kStageBytes;
            uint8_t *sb = sa + kBytesA;
            mbar_expect_tx(&full_bar[s], args.gather ? kBytesB : kStageBytes);
            const int kx = kblock_offset(args, kb, k_begin, cls);
            if (!args.gather) tma_load_2d(sa, &map_a, &full_bar[s], kx, m0);
            tma_load_2d(sb, &map_b, &full_bar[s], kx, n0);
        }
        issued_kb = kb;
    } else if (warp == 1 && lane == 0) {
        // MMA issuer.
        constexpr uint32_t idesc = instr_desc(kBM, BN);
        int kb = 0;
        for (; kb < num_kb; ++kb) {
            const int s = kb % nst;
            if (!mbar_wait(&full_bar[s], (kb / nst) & 1)) {
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
        // Operand A producers: kGatherThreads threads, thread g copies chunk
        // j = g % 8 of rows g / 8 + (kGatherThreads / 8) i of the 128 x 64
        // tile, so eight threads read one row's 128 contiguous bytes (one
        // tap, or two for C = 32).
        // Row r, chunk j lands at byte r * 128 + ((j ^ (r % 8)) * 16) of the
        // 1024-byte-aligned stage, the 128-byte swizzle of the TMA loads it
        // replaces.  Each stage's copies form one cp.async group; a warp
        // keeps up to kAhead groups in flight.  At the top of each iteration
        // the oldest group is waited for, fenced to the async proxy that
        // tcgen05.mma reads through and arrived on its full barrier, before
        // the warp waits for the next ring slot, so the slot's release (by
        // the MMAs of a stage arrived kAhead iterations earlier) is never
        // held up by the warp's own arrivals.
        // kAhead <= ring depth: the slot waited for at iteration kb belongs to
        // stage kb - nst, arrived at the top of iteration kb - nst + kAhead <= kb.
        constexpr int kAhead = GBDIC_GATHER_AHEAD;
        static_assert(kAhead >= 1 && kAhead <= kGatherStages, "gather look-ahead must stay within the ring");
        constexpr int kRowStep = kGatherThreads / 8, kRowsPerThread = kBM / kRowStep;
        const int g = tid - 64, j = g & 7, r0 = g >> 3;
        int kb = 0, arrived = 0;
        for (; kb < num_kb; ++kb) {
            const int s = kb % nst;
            if (kb - arrived == kAhead) {
                asm volatile("cp.async.wait_group %0;" ::"n"(kAhead - 1) : "memory");
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&full_bar[arrived % nst]);
                ++arrived;
            }
            if (kb >= nst) {
                int ok = 1;
                if (lane == 0) ok = mbar_wait(&empty_bar[s], ((kb / nst) - 1) & 1) ? 1 : 0;
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) {
                    if (lane == 0) atomicExch(&failed, 1);
                    break;
                }
            }
            const uint32_t sa = smem_u32(smem + s * kStageBytes);
            const int4 tap = gather_tap(args, kblock_offset(args, kb, k_begin, cls) + 8 * j, cls);
#pragma unroll
            for (int i = 0; i < kRowsPerThread; ++i) {
                const int r = r0 + kRowStep * i;
                const uint4 *src = gather_src(args, row_tab[r], tap);
                cp_async_16(sa + (uint32_t)(r * 128 + ((j ^ (r & 7)) << 4)), src ? src : args.a, src ? 16u : 0u);
            }
            asm volatile("cp.async.commit_group;" ::: "memory");
        }
        // Drain: every issued copy lands before the warp moves on (also after
        // a failed wait, so no copy is left writing into shared memory).
        asm volatile("cp.async.wait_all;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        for (; arrived < kb; ++arrived)
            if (lane == 0) mbar_arrive(&full_bar[arrived % nst]);
    }
    __syncwarp();
    if (!mbar_wait(&done_bar, 0)) atomicExch(&failed, 1);
    __syncwarp();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    // Epilogue: warp w < 4 owns accumulator lanes (rows) 32w .. 32w + 31.
    const int row = output_row(args, m0 + warp * 32 + lane, cls);
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll 1
    for (int c = 0; c < (warp < 4 ? BN : 0); c += 16) {
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
            for (int kb = consumed_kb; kb < issued_kb; ++kb) mbar_wait(&full_bar[kb % nst], (kb / nst) & 1);
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
    const int num_kb = a.K / a.k_split / kBK;
    const int ring = a.gather ? kGatherStages : kStages;
    const int nst = num_kb < ring ? num_kb : ring;
    const size_t smem = (size_t)nst * (kBM * kBK * 2 + BN * kBK * 2) + 1024;
    const size_t smem_max = (size_t)kStages * (kBM * kBK * 2 + BN * kBK * 2) + 1024;
    // The attribute is per device; set it once per device and tile width.
    static thread_local int configured_device = -1;
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err != cudaSuccess) return err;
    if (configured_device != device) {
        err = cudaFuncSetAttribute(tc_gemm_kernel<BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        if (err != cudaSuccess) return err;
        configured_device = device;
    }
    dim3 grid(a.N / BN, a.M / kBM, a.k_split);
    tc_gemm_kernel<BN><<<grid, a.gather ? kMaxThreads : 128, smem, stream>>>(ma, mb, a);
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
        // k_split > 1 (partials per split, as for a plain GEMM) for the
        // im2col gather only.
        const NnConvShape &s = a.conv;
        if ((a.k_split != 1 && a.gather != kGatherIm2col) || s.B < 1 || s.H < 1 || s.W < 1 ||
            s.OH != (s.H + 1) / 2 || s.OW != (s.W + 1) / 2)
            return cudaErrorInvalidValue;
        // chunk offsets are 32-bit in the kernel
        if (a.gather == kGatherIm2col) {
            if (s.C < 8 || s.C % 8 || a.M != s.B * s.OH * s.OW || a.K != s.Kp || s.Kp < 9 * s.C ||
                (long long)s.B * s.H * s.W * (s.C / 8) >= (1ll << 31))
                return cudaErrorInvalidValue;
        } else if (a.gather == kGatherDgrad) {
            if (s.Cout < 8 || s.Cout % 8 || a.M != s.B * s.H * s.W || a.K != 9 * s.Cout ||
                (long long)s.B * s.OH * s.OW * (s.Cout / 8) >= (1ll << 31))
                return cudaErrorInvalidValue;
        } else {
            return cudaErrorInvalidValue;
        }
    }
    TcGemmArgs args = a;
    if (a.gather == kGatherDgrad) {
        // Rows by parity class, zero taps skipped: same sums (the skipped K
        // blocks are exact zeros), a quarter of the gathers and MMAs.
        const NnConvShape &s = a.conv;
        if (s.H == 2 * s.OH && s.W == 2 * s.OW && s.Cout % kBK == 0 && (s.B * s.OH * s.OW) % kBM == 0)
            args.gather = kGatherDgradClasses;
    } else if (a.gather != kGatherNone && a.gather != kGatherIm2col) {
        return cudaErrorInvalidValue;
    }
    CUtensorMap ma, mb;
    if (!make_map(&mb, args.b, args.N, args.K, bn)) return cudaErrorInvalidValue;
    if (args.gather == kGatherNone) {
        if (!make_map(&ma, args.a, args.M, args.K, kBM)) return cudaErrorInvalidValue;
    } else {
        ma = mb;  // not read: operand A is gathered
    }
    switch (bn) {
    case 128: return launch_bn<128>(ma, mb, args, stream);
    case 64: return launch_bn<64>(ma, mb, args, stream);
    case 32: return launch_bn<32>(ma, mb, args, stream);
    default: return launch_bn<16>(ma, mb, args, stream);
    }
}

}  // namespace gbdic
