// tc_gemm.cuh -- FP32-accumulating TF32 GEMM on the 5th-generation tensor
// cores: C[M x N] = A[M x K] * B[N x K]^T, A and B K-major in global memory.
//
// One CTA computes a 128 x 128 tile of C:
//   * thread 0 streams 128 x 32 tiles of A and B (128-byte rows) by TMA
//     (cp.async.bulk.tensor.2d, 128-byte swizzle) into a ring of NSTAGE stages
//     guarded by "full" mbarriers;
//   * thread 32 issues tcgen05.mma (kind::tf32, M = 128, N = 128, K = 8 per
//     instruction, four per 32-wide K chunk) accumulating into 128 TMEM
//     columns, and tcgen05.commit releases each stage through its "empty"
//     mbarrier once the MMAs that read it have completed;
//   * after the last commit, the four warps read their 32 TMEM lanes (rows)
//     with tcgen05.ld and store the tile.
// Two CTAs share an SM (3 stages, 128 of the SM's 512 TMEM columns each), so
// one CTA's MMAs overlap the other's epilogue and set-up.
// Every wait is bounded (2 s of %globaltimer); on expiry the CTA sets *err,
// waits (bounded) for the copies and MMAs it issued, frees its TMEM and returns.
//
// The caller pads M and N to multiples of 128 and K to a multiple of 32 with
// zeros, and stores TF32-representable values (low 13 mantissa bits zero), so
// the tensor cores see exactly the values given.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace mfdtd {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 32;          // tile; BK fp32 = one 128-byte row
constexpr int NSTAGE = 3;                           // 3 x 32 KB: two CTAs fit on one SM
constexpr int TILE_B = BM * BK * 4;                 // 16 KB per operand tile
constexpr int STAGE_BYTES = 2 * TILE_B;             // A + B
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + 1024 /* alignment */ + 256 /* barriers */;
constexpr int THREADS = 128;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void bar_init(uint64_t *b, unsigned n) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(n) : "memory");
}
__device__ __forceinline__ bool bar_test(uint64_t *b, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool bar_wait(uint64_t *b, unsigned parity) {
    if (bar_test(b, parity)) return true;
    const uint64_t t0 = gtimer();
    for (;;) {
        if (bar_test(b, parity)) return true;
        if (gtimer() - t0 > 2000000000ull) return false;
    }
}

// Shared-memory matrix descriptor of a K-major tile with 128-byte swizzling:
// start address >> 4 (bits 0-13), leading-dimension offset unused for this
// layout (1), stride between 8-row groups 1024 B >> 4 (bits 32-45), the fixed
// value 0b001 at bits 46-48, base offset 0 (tile 1024-byte aligned), swizzle
// mode 2 = 128-byte (bits 61-63).
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor, kind::tf32: D = F32 (bits 4-5 = 1), A = B = TF32
// (bits 7-9, 10-12 = 2), both K-major (bits 15, 16 = 0), N >> 3 at bits
// 17-22, M >> 4 at bits 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) |
                            ((uint32_t)(BM >> 4) << 24);

__global__ void __launch_bounds__(THREADS, 2)
    k_tc_gemm_tf32(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   float *__restrict__ C, int ldc, int nk, unsigned int *err) {
    extern __shared__ __align__(1024) unsigned char raw[];
    unsigned char *base = raw + ((1024u - (smem_addr(raw) & 1023u)) & 1023u);
    uint64_t *full = (uint64_t *)(base + NSTAGE * STAGE_BYTES);
    uint64_t *empty = full + NSTAGE;
    uint64_t *done = empty + NSTAGE;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; s++) {
            bar_init(&full[s], 1);
            bar_init(&empty[s], 1);
        }
        bar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {  // 128 TMEM columns: the 128 x 128 FP32 accumulator
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_addr(tmem_slot)),
                     "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;
    __shared__ int s_fail;
    if (tid == 0) s_fail = 0;
    __syncthreads();

    int issued = 0;     // TMA stages issued (producer)
    if (tid == 0) {
        // producer
        for (int kc = 0; kc < nk; kc++) {
            const int s = kc % NSTAGE;
            if (kc >= NSTAGE && !bar_wait(&empty[s], ((kc / NSTAGE) - 1) & 1)) {
                s_fail = 1;
                break;
            }
            unsigned char *sa = base + s * STAGE_BYTES, *sb = sa + TILE_B;
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&full[s])),
                         "r"(STAGE_BYTES)
                         : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
                "{%2, %3}], [%4];" ::"r"(smem_addr(sa)),
                "l"((uint64_t)&mapA), "r"(kc * BK), "r"(m0), "r"(smem_addr(&full[s]))
                : "memory");
            asm volatile(
                "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
                "{%2, %3}], [%4];" ::"r"(smem_addr(sb)),
                "l"((uint64_t)&mapB), "r"(kc * BK), "r"(n0), "r"(smem_addr(&full[s]))
                : "memory");
            issued = kc + 1;
        }
    } else if (tid == 32) {
        // MMA issuer
        for (int kc = 0; kc < nk; kc++) {
            const int s = kc % NSTAGE;
            if (!bar_wait(&full[s], (kc / NSTAGE) & 1)) {
                s_fail = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t sa = smem_addr(base + s * STAGE_BYTES), sb = sa + TILE_B;
#pragma unroll
            for (int kk = 0; kk < BK / 8; kk++) {  // K = 8 TF32 = 32 bytes per instruction
                const uint64_t da = sw128_desc(sa + kk * 32), db = sw128_desc(sb + kk * 32);
                const uint32_t acc = (kc > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.u32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(kIdesc), "r"(acc)
                    : "memory");
            }
            // the stage is free once these MMAs have read it
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&empty[s]))
                         : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_addr(done))
                     : "memory");
    }
    // everyone waits for the accumulator (bounded)
    bool ok = bar_wait(done, 0);
    __syncthreads();
    if (s_fail || !ok) {
        if (tid == 0) atomicOr(err, 1u);
        if (tid == 0)  // let issued copies land before the CTA's shared memory goes away
            for (int kc = 0; kc < issued; kc++) {
                const uint64_t t0 = gtimer();
                while (!bar_test(&full[kc % NSTAGE], (kc / NSTAGE) & 1) && gtimer() - t0 < 200000000ull) {
                }
            }
    } else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // warp w owns TMEM lanes 32w..32w+31 = rows m0 + 32w + lane
        const int row = m0 + warp * 32 + (tid & 31);
#pragma unroll
        for (int c0 = 0; c0 < BN; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
                "%11, %12, %13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]),
                  "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]),
                  "=r"(v[14]), "=r"(v[15])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float *dst = C + (size_t)row * ldc + n0 + c0;
#pragma unroll
            for (int q = 0; q < 16; q += 4)
                *(float4 *)(dst + q) = make_float4(__uint_as_float(v[q]), __uint_as_float(v[q + 1]),
                                                   __uint_as_float(v[q + 2]), __uint_as_float(v[q + 3]));
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN) : "memory");
}

}  // namespace tc
}  // namespace mfdtd
