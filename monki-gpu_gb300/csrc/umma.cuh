// Fifth-generation tensor-core GEMM for sm_103a: C = A * B^T with BF16 operands staged
// in shared memory (128-byte swizzled, K-major), FP32 accumulation in tensor memory
// (TMEM), one elected thread issuing tcgen05.mma, completion tracked by mbarriers, and a
// fused epilogue read back from TMEM with tcgen05.ld.
//
// Tile: 128 rows of C per CTA (the MMA's M), all N <= 256 columns (one MMA covers them),
// K in steps of 64 (one 128-byte swizzle row of BF16), four MMAs of K = 16 per step.
// Two shared-memory stages: the 256 threads load step s + 1 while the tensor core runs
// step s; a stage is refilled only after the MMAs that read it have committed. The K
// range of a CTA is blockIdx.y's slice (split-K for the weight gradients).
//
// Shared-memory matrix layout (K-major, SWIZZLE_128B): row r of a tile occupies bytes
// [128 r, 128 r + 128); its 16-byte chunk c sits at chunk c ^ (r % 8). Eight rows form a
// 1024-byte atom, so the descriptor's stride byte offset is 1024 and the tile base is
// 1024-byte aligned. Advancing the start address by 32 bytes selects the next K = 16.
#pragma once
#include <stdint.h>
#include <cuda_bf16.h>

namespace monki {
namespace umma {

constexpr int kBlockM = 128;
constexpr int kBlockK = 64;
constexpr int kThreads = 256;                    // eight warps: loaders, then epilogue
constexpr uint32_t kSmemA = kBlockM * kBlockK * 2;   // 16 KB
constexpr uint32_t kSmemB = 256 * kBlockK * 2;       // 32 KB (N <= 256)
constexpr uint32_t kStage = kSmemA + kSmemB;         // 48 KB, 1024-byte multiple
// 100 KB of dynamic shared memory: two stages plus alignment, and at most two CTAs per SM
// so their TMEM allocations (256 columns each of the SM's 512) never wait on each other.
constexpr uint32_t kSmemBytes = 100u * 1024u;
constexpr uint32_t kWaitLimit = 1u << 24;          // mbarrier polls before giving up

enum Epilogue : int {
    kStore = 0,      // C (fp32) = acc
    kForward = 1,    // Z (fp32) = acc + bias; H (bf16) = GELU(Z); H^T (bf16)
    kBackward = 2,   // G = acc * GELU'(Zprev); G (bf16) and G^T (bf16)
    kAccumulate = 3, // C (fp32) += acc (split-K partial, atomics)
};

struct Params {
    const __nv_bfloat16* A;   // rows_a x K, row stride lda (elements)
    const __nv_bfloat16* B;   // N x K, row stride ldb
    int rows_a, N, K, lda, ldb;
    int k_chunk;              // K elements per blockIdx.y slice (multiple of 64)
    float* C;                 // kStore / kAccumulate / kForward (Z): rows_a x N, stride N
    const float* bias;        // kForward: N
    const float* zprev;       // kBackward: rows_a x N pre-activations
    __nv_bfloat16* H;         // kForward / kBackward: rows_a x N
    __nv_bfloat16* HT;        // kForward / kBackward: N x rows_ht (transposed), or null
    int rows_ht;              // row stride of HT (>= rows_a)
    uint32_t* failure;        // bit 1: an mbarrier wait gave up
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor: start address, leading byte offset (unused by the
// swizzled K-major layout, 16 bytes), stride byte offset 1024, descriptor version 1,
// layout SWIZZLE_128B (2).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
    uint64_t d = 0;
    d |= uint64_t((addr & 0x3FFFFu) >> 4);
    d |= uint64_t(16u >> 4) << 16;
    d |= uint64_t(1024u >> 4) << 32;
    d |= uint64_t(1) << 46;
    d |= uint64_t(2) << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major.
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(n >> 3) << 17) | (uint32_t(m >> 4) << 24);
}

__device__ __forceinline__ float gelu(float z) {
    return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
    const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
    const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
    return cdf + z * pdf;
}

// Copy rows [row0, row0 + rows) x columns [k0, k0 + 64) of a K-major BF16 matrix into a
// swizzled tile; rows past `limit` are zero.
__device__ __forceinline__ void load_tile(unsigned char* tile, const __nv_bfloat16* g, int ld, int row0, int rows,
                                          int limit, int k0) {
    const int chunks = rows * 8;
    for (int q = threadIdx.x; q < chunks; q += kThreads) {
        const int r = q >> 3, c = q & 7;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (row0 + r < limit)
            v = *reinterpret_cast<const uint4*>(g + size_t(row0 + r) * ld + k0 + c * 8);
        *reinterpret_cast<uint4*>(tile + r * 128 + ((c ^ (r & 7)) << 4)) = v;
    }
}

__device__ __forceinline__ bool wait_parity(uint32_t bar, uint32_t parity) {
    for (uint32_t attempt = 0; attempt < kWaitLimit; ++attempt) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}"
            : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

template <int EPI>
__global__ void __launch_bounds__(kThreads, 1) gemm(Params p) {
    extern __shared__ __align__(1024) unsigned char raw[];
    __shared__ __align__(8) uint64_t mma_bar[2];
    __shared__ uint32_t tmem_base;
    __shared__ int aborted;
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * kBlockM;
    const int k_begin = blockIdx.y * p.k_chunk;
    const int k_end = min(p.K, k_begin + p.k_chunk);
    const int N = p.N;
    const uint32_t columns = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
    const uint32_t bar[2] = {smem_u32(&mma_bar[0]), smem_u32(&mma_bar[1])};

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(columns) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        aborted = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar[0]) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar[1]) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;
    const uint32_t idesc = instr_desc(kBlockM, N);

    // Commits issued and completions observed per stage barrier (uniform in the CTA).
    uint32_t issued[2] = {0u, 0u}, seen[2] = {0u, 0u};
    int step = 0;
    for (int k0 = k_begin; k0 < k_end; k0 += kBlockK, ++step) {
        const int b = step & 1;
        unsigned char* tile_a = base + b * kStage;
        unsigned char* tile_b = tile_a + kSmemA;
        if (issued[b] > seen[b]) {
            // The MMAs of step - 2 read this stage: wait for their commit before refilling.
            if (!wait_parity(bar[b], seen[b] & 1u)) {
                aborted = 1;
                if (threadIdx.x == 0) atomicOr(p.failure, 1u);
            }
            ++seen[b];
        }
        load_tile(tile_a, p.A, p.lda, row0, kBlockM, p.rows_a, k0);
        load_tile(tile_b, p.B, p.ldb, 0, N, N, k0);
        // Make the generic-proxy stores visible to the tensor core (async proxy).
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (aborted) break;
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_addr = smem_u32(tile_a), b_addr = smem_u32(tile_b);
#pragma unroll
            for (int kk = 0; kk < kBlockK / 16; ++kk) {
                const uint64_t da = smem_desc(a_addr + kk * 32), db = smem_desc(b_addr + kk * 32);
                const uint32_t accumulate = (k0 > k_begin || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(accumulate) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar[b])
                         : "memory");
        }
        ++issued[b];
    }
    // Drain: every commit issued is waited for (bounded) before TMEM is read or released.
    for (int b = 0; b < 2; ++b) {
        while (seen[b] < issued[b]) {
            if (!wait_parity(bar[b], seen[b] & 1u)) {
                aborted = 1;
                if (threadIdx.x == 0) atomicOr(p.failure, 1u);
            }
            ++seen[b];
        }
    }
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (!aborted && k_end > k_begin) {
        // Epilogue: warp w reads TMEM lanes (rows) 32 (w % 4) .. + 31 (the lane quarter its
        // position in the warpgroup allows) and every other 32-column chunk, from 32 (w / 4).
        const int quarter = warp & 3, half = warp >> 2;
        const int m = row0 + quarter * 32 + lane;
        const bool valid = m < p.rows_a;
        for (int c0 = 32 * half; c0 < N; c0 += 64) {
            uint32_t r[32];
            const uint32_t taddr = tmem + (uint32_t(quarter * 32) << 16) + uint32_t(c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
                "%14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
                  "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                  "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!valid) continue;
            const int width = min(32, N - c0);
            const size_t at = size_t(m) * N + c0;
            // Each thread owns 32 consecutive columns of its row: 16-byte stores (and loads)
            // instead of scalar ones, whose warp-wide pattern touched 32 rows per instruction.
            if (width == 32 && (N & 7) == 0) {
                float v[32];
#pragma unroll
                for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
                if (EPI == kStore) {
#pragma unroll
                    for (int q = 0; q < 32; q += 4)
                        *reinterpret_cast<float4*>(p.C + at + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                } else if (EPI == kAccumulate) {
#pragma unroll
                    for (int q = 0; q < 32; q += 4)
                        atomicAdd(reinterpret_cast<float4*>(p.C + at + q), make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]));
                } else {
                    if (EPI == kForward) {
#pragma unroll
                        for (int q = 0; q < 32; q += 4) {
                            const float4 b = *reinterpret_cast<const float4*>(p.bias + c0 + q);
                            v[q] += b.x; v[q + 1] += b.y; v[q + 2] += b.z; v[q + 3] += b.w;
                            *reinterpret_cast<float4*>(p.C + at + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                        }
#pragma unroll
                        for (int q = 0; q < 32; ++q) v[q] = gelu(v[q]);
                    } else {
#pragma unroll
                        for (int q = 0; q < 32; q += 4) {
                            const float4 z = *reinterpret_cast<const float4*>(p.zprev + at + q);
                            v[q] *= gelu_grad(z.x); v[q + 1] *= gelu_grad(z.y);
                            v[q + 2] *= gelu_grad(z.z); v[q + 3] *= gelu_grad(z.w);
                        }
                    }
                    uint32_t packed[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                        packed[q] = *reinterpret_cast<const uint32_t*>(&h2);
                    }
#pragma unroll
                    for (int q = 0; q < 16; q += 4)
                        *reinterpret_cast<uint4*>(p.H + at + 2 * q) = make_uint4(packed[q], packed[q + 1], packed[q + 2], packed[q + 3]);
                    if (p.HT) {
#pragma unroll
                        for (int q = 0; q < 32; ++q)
                            p.HT[size_t(c0 + q) * p.rows_ht + m] = __float2bfloat16(v[q]);
                    }
                }
                continue;
            }
#pragma unroll
            for (int q = 0; q < 32; ++q) {
                if (q >= width) break;
                const int n = c0 + q;
                const float acc = __uint_as_float(r[q]);
                const size_t e = size_t(m) * N + n;
                if (EPI == kStore) {
                    p.C[e] = acc;
                } else if (EPI == kAccumulate) {
                    atomicAdd(p.C + e, acc);
                } else if (EPI == kForward) {
                    const float z = acc + p.bias[n];
                    p.C[e] = z;
                    const __nv_bfloat16 h = __float2bfloat16(gelu(z));
                    p.H[e] = h;
                    if (p.HT) p.HT[size_t(n) * p.rows_ht + m] = h;
                } else {
                    const __nv_bfloat16 g = __float2bfloat16(acc * gelu_grad(p.zprev[e]));
                    p.H[e] = g;
                    if (p.HT) p.HT[size_t(n) * p.rows_ht + m] = g;
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(columns) : "memory");
}

}  // namespace umma
}  // namespace monki
