// Fifth-generation tensor-core GEMM for sm_103a: C = A * B^T with BF16 operands, FP32
// accumulation in tensor memory (TMEM) and a fused epilogue read back with tcgen05.ld.
//
// Roles inside a CTA of eight warps:
//   producer  (warp 0, one thread) loads the K-steps' A and B tiles with the Tensor Memory
//             Accelerator (cp.async.bulk.tensor, 128-byte swizzle) into a ring of shared-
//             memory stages (two; four for the split-K weight gradients, one CTA per SM);
//             each load completes on the stage's "full" mbarrier;
//   MMA       (warp 1, one thread) waits for a stage, issues four tcgen05.mma of K = 16 and
//             commits them to the stage's "empty" mbarrier, which frees it for the next
//             load; the last commit also arrives on the "done" mbarrier;
//   epilogue  (all eight warps) after "done": TMEM lanes 32 (w % 4) .. + 31, every other
//             32-column chunk from 32 (w / 4); bias, GELU or GELU', FP32 / BF16 stores, and
//             transposed BF16 stores staged through shared memory so that each thread
//             writes 64 contiguous bytes of a transposed row (and, in the backward
//             epilogue, adds that row's 32 values to the column's bias gradient).
//
// Tile: 128 rows of C per CTA (the MMA's M), all N <= 256 columns (one MMA covers them),
// K in steps of 64 (one 128-byte swizzle row of BF16). The K range of a CTA is blockIdx.y's
// slice (split-K for the weight gradients, summed by float4 atomics). Every mbarrier wait is
// bounded: a wait that gives up sets failure bit 1, the CTA skips its stores and still
// releases its TMEM.
//
// Shared-memory operand layout (K-major, SWIZZLE_128B, what the TMA writes with
// CU_TENSOR_MAP_SWIZZLE_128B): row r of a tile occupies bytes [128 r, 128 r + 128); its
// 16-byte chunk c sits at chunk c ^ (r % 8). Eight rows form a 1024-byte atom, so the
// descriptor's stride byte offset is 1024 and each tile base is 1024-byte aligned.
// Advancing the start address by 32 bytes selects the next K = 16.
#pragma once
#include <stdint.h>
#include <cuda.h>
#include <cuda_bf16.h>

namespace monki {
namespace umma {

constexpr int kBlockM = 128;
constexpr int kBlockK = 64;
constexpr int kThreads = 256;                    // eight warps
constexpr int kStages = 2;                       // shared-memory stages of the output-tile GEMMs
constexpr uint32_t kSmemA = kBlockM * kBlockK * 2;   // 16 KB
constexpr uint32_t kSmemB = 256 * kBlockK * 2;       // 32 KB (N <= 256)
constexpr uint32_t kStage = kSmemA + kSmemB;         // 48 KB, 1024-byte multiple
// 100 KB of dynamic shared memory: the stages plus alignment, so two CTAs share an SM and
// their TMEM allocations (256 columns each of the SM's 512) never wait on each other.
constexpr uint32_t kSmemBytes = 100u * 1024u;
constexpr uint32_t kWaitLimit = 1u << 24;          // mbarrier polls before giving up
constexpr uint32_t kTransposeStride = 80;          // bytes per staged transposed row (32 BF16 + padding)

enum Epilogue : int {
    kStore = 0,      // C (fp32) = acc
    kForward = 1,    // Z (bf16) = acc + bias; H (bf16) = GELU(Z); H^T (bf16)
    kBackward = 2,   // G = acc * GELU'(Zprev); G (bf16), G^T (bf16), column sums of G
    kAccumulate = 3, // C (fp32) += acc (split-K partial, atomics)
};

// The split-K weight-gradient GEMM runs one CTA per SM (its grid is about one wave) over 16
// K steps, so it keeps four stages in flight instead of two.
constexpr int kAccumulateStages = 4;
template <int EPI>
constexpr int stages_of() { return EPI == kAccumulate ? kAccumulateStages : kStages; }
template <int EPI>
constexpr uint32_t smem_bytes_of() { return EPI == kAccumulate ? uint32_t(kAccumulateStages) * (kSmemA + kSmemB) + 4096u : kSmemBytes; }

struct Params {
    int rows_a, N, K;
    int k_chunk;              // K elements per blockIdx.y slice (multiple of 64)
    float* C;                 // kStore / kAccumulate: rows_a x N, stride N
    __nv_bfloat16* Z;         // kForward: rows_a x N pre-activations (BF16)
    const float* bias;        // kForward: N
    const __nv_bfloat16* zprev;  // kBackward: rows_a x N pre-activations (BF16)
    float* bias_grad;         // kBackward: N column sums of G are added here (needs HT), or null
    __nv_bfloat16* H;         // kForward / kBackward: rows_a x N
    __nv_bfloat16* HT;        // kForward / kBackward: N x rows_ht (transposed), or null
    int rows_ht;              // row stride of HT (>= rows_a, a multiple of 8)
    // kForward, optional: a linear output layer on the BF16 activations, y = H head_w +
    // head_b[0] per row (head_w: N values), written to head_y (rows_a values).
    const float* head_w;
    const float* head_b;
    float* head_y;
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

// One 2-D tile (x = K element, y = row) of a tensor map into shared memory, completing
// `bytes` on the mbarrier.
__device__ __forceinline__ void tma_load(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar) : "memory");
}

template <int EPI>
__global__ void __launch_bounds__(kThreads, 1)
gemm(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, Params p) {
    extern __shared__ __align__(1024) unsigned char raw[];
    constexpr int kRing = stages_of<EPI>();
    __shared__ __align__(8) uint64_t full_bar[kRing], empty_bar[kRing], done_bar;
    __shared__ uint32_t tmem_base;
    __shared__ int aborted;
    __shared__ int issued, consumed;  // K steps whose loads were issued / whose MMAs were committed
    unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row0 = blockIdx.x * kBlockM;
    const int k_begin = blockIdx.y * p.k_chunk;
    const int k_end = min(p.K, k_begin + p.k_chunk);
    const int steps = k_end > k_begin ? (k_end - k_begin) / kBlockK : 0;
    const int N = p.N;
    const uint32_t columns = N <= 32 ? 32u : (N <= 64 ? 64u : (N <= 128 ? 128u : 256u));
    const uint32_t b_rows = uint32_t(N);  // the B tile's rows (the tensor map's box height)
    const uint32_t stage_bytes = kSmemA + b_rows * kBlockK * 2;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(columns) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 32) {
        aborted = 0;
        issued = 0;
        consumed = 0;
        for (int s = 0; s < kRing; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&full_bar[s])) : "memory");
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&empty_bar[s])) : "memory");
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&done_bar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base;

    if (threadIdx.x == 0 && steps > 0) {
        // Producer: a stage is reloaded only after the MMAs that read it have committed.
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_a)) : "memory");
        asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&map_b)) : "memory");
        for (int step = 0; step < steps; ++step) {
            const int s = step % kRing, round = step / kRing;
            if (round > 0 && !wait_parity(smem_u32(&empty_bar[s]), uint32_t(round - 1) & 1u)) {
                atomicOr(p.failure, 1u);
                aborted = 1;
                break;
            }
            const uint32_t full = smem_u32(&full_bar[s]);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full), "r"(stage_bytes) : "memory");
            const uint32_t tile_a = smem_u32(base + s * kStage), tile_b = tile_a + kSmemA;
            const int k0 = k_begin + step * kBlockK;
            tma_load(tile_a, &map_a, k0, row0, full);
            tma_load(tile_b, &map_b, k0, 0, full);
            issued = step + 1;
        }
    } else if (threadIdx.x == 32 && steps > 0) {
        // MMA issuer.
        const uint32_t idesc = instr_desc(kBlockM, N);
        for (int step = 0; step < steps; ++step) {
            const int s = step % kRing, round = step / kRing;
            if (!wait_parity(smem_u32(&full_bar[s]), uint32_t(round) & 1u)) {
                atomicOr(p.failure, 1u);
                aborted = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_addr = smem_u32(base + s * kStage), b_addr = a_addr + kSmemA;
#pragma unroll
            for (int kk = 0; kk < kBlockK / 16; ++kk) {
                const uint64_t da = smem_desc(a_addr + kk * 32), db = smem_desc(b_addr + kk * 32);
                const uint32_t accumulate = (step > 0 || kk > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}"
                    ::"r"(tmem), "l"(da), "l"(db), "r"(idesc), "r"(accumulate) : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(smem_u32(&empty_bar[s])) : "memory");
            consumed = step + 1;
        }
        // Every MMA issued so far completes before "done" arrives.
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                     ::"r"(smem_u32(&done_bar)) : "memory");
    }
    __syncwarp();
    if (steps > 0 && !wait_parity(smem_u32(&done_bar), 0u)) {
        if (lane == 0) atomicOr(p.failure, 1u);
        aborted = 1;
    }
    // The producer's loads were all consumed by MMAs that "done" covers; the stages are free.
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (aborted && threadIdx.x == 0) {
        // A wait gave up: the loads issued but never consumed may still be in flight. Wait for
        // them (each wait bounded) before the block ends and its shared memory is reused.
        for (int step = consumed; step < issued; ++step)
            wait_parity(smem_u32(&full_bar[step % kRing]), uint32_t(step / kRing) & 1u);
    }

    // The output layer's partial sums of each row (two halves of the columns), after the
    // transpose tiles.
    float* head_part = reinterpret_cast<float*>(base + 32 * 1024);
    if (!aborted && steps > 0) {
        const int quarter = warp & 3, half = warp >> 2;
        const int m = row0 + quarter * 32 + lane;
        const bool valid = m < p.rows_a;
        float head = 0.f;
        unsigned char* stage_t = base + warp * (32 * kTransposeStride);  // this warp's transpose tile
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
            const int width = min(32, N - c0);
            const size_t at = size_t(m) * N + c0;
            if (width == 32 && (N & 7) == 0) {
                float v[32];
#pragma unroll
                for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
                if (EPI == kStore) {
                    if (valid)
#pragma unroll
                        for (int q = 0; q < 32; q += 4)
                            *reinterpret_cast<float4*>(p.C + at + q) = make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]);
                } else if (EPI == kAccumulate) {
                    if (valid)
#pragma unroll
                        for (int q = 0; q < 32; q += 4)
                            atomicAdd(reinterpret_cast<float4*>(p.C + at + q), make_float4(v[q], v[q + 1], v[q + 2], v[q + 3]));
                } else {
                    if (EPI == kForward) {
                        uint32_t zp[16];
#pragma unroll
                        for (int q = 0; q < 32; q += 4) {
                            const float4 b = *reinterpret_cast<const float4*>(p.bias + c0 + q);
                            v[q] += b.x; v[q + 1] += b.y; v[q + 2] += b.z; v[q + 3] += b.w;
                        }
#pragma unroll
                        for (int q = 0; q < 16; ++q) {
                            const __nv_bfloat162 z2 = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                            zp[q] = *reinterpret_cast<const uint32_t*>(&z2);
                        }
                        if (valid)
#pragma unroll
                            for (int q = 0; q < 16; q += 4)
                                *reinterpret_cast<uint4*>(p.Z + at + 2 * q) = make_uint4(zp[q], zp[q + 1], zp[q + 2], zp[q + 3]);
#pragma unroll
                        for (int q = 0; q < 32; ++q) v[q] = gelu(v[q]);
                    } else if (valid) {
                        // GELU' of the stored (BF16) pre-activations.
#pragma unroll
                        for (int q = 0; q < 32; q += 8) {
                            const uint4 z8 = *reinterpret_cast<const uint4*>(p.zprev + at + q);
                            const uint32_t zw[4] = {z8.x, z8.y, z8.z, z8.w};
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                const float2 z2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&zw[u]));
                                v[q + 2 * u] *= gelu_grad(z2.x);
                                v[q + 2 * u + 1] *= gelu_grad(z2.y);
                            }
                        }
                    }
                    uint32_t packed[16];
#pragma unroll
                    for (int q = 0; q < 16; ++q) {
                        const __nv_bfloat162 h2 = __floats2bfloat162_rn(v[2 * q], v[2 * q + 1]);
                        packed[q] = *reinterpret_cast<const uint32_t*>(&h2);
                    }
                    if (valid)
#pragma unroll
                        for (int q = 0; q < 16; q += 4)
                            *reinterpret_cast<uint4*>(p.H + at + 2 * q) =
                                make_uint4(packed[q], packed[q + 1], packed[q + 2], packed[q + 3]);
                    if (EPI == kForward && p.head_w) {
#pragma unroll
                        for (int q = 0; q < 16; q += 2) {
                            const float4 w = *reinterpret_cast<const float4*>(p.head_w + c0 + 2 * q);
                            const float2 h0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&packed[q]));
                            const float2 h1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&packed[q + 1]));
                            head += h0.x * w.x + h0.y * w.y + h1.x * w.z + h1.y * w.w;
                        }
                    }
                    if (p.HT) {
                        // Transpose through shared memory: lane (row m) writes its 32 values down
                        // a column of the warp's tile, then lane (column c0 + lane) writes the 32
                        // rows of its column as 64 contiguous bytes.
                        __nv_bfloat16* tile = reinterpret_cast<__nv_bfloat16*>(stage_t);
#pragma unroll
                        for (int q = 0; q < 32; ++q)
                            tile[q * (kTransposeStride / 2) + lane] = valid ? __float2bfloat16(v[q]) : __float2bfloat16(0.f);
                        __syncwarp();
                        const int m0 = row0 + quarter * 32;
                        const uint4* row = reinterpret_cast<const uint4*>(stage_t + lane * kTransposeStride);
                        __nv_bfloat16* dst = p.HT + size_t(c0 + lane) * p.rows_ht + m0;
                        if (m0 + 32 <= p.rows_ht) {
#pragma unroll
                            for (int q = 0; q < 4; ++q) reinterpret_cast<uint4*>(dst)[q] = row[q];
                        } else {
                            const __nv_bfloat16* src = reinterpret_cast<const __nv_bfloat16*>(row);
                            for (int q = 0; m0 + q < p.rows_ht; ++q) dst[q] = src[q];
                        }
                        if (EPI == kBackward && p.bias_grad) {
                            // Column c0 + lane of G over this warp's 32 rows (rows past rows_a
                            // were staged as zeros).
                            const __nv_bfloat162* g2 = reinterpret_cast<const __nv_bfloat162*>(row);
                            float sum = 0.f;
#pragma unroll
                            for (int q = 0; q < 16; ++q) {
                                const float2 f = __bfloat1622float2(g2[q]);
                                sum += f.x + f.y;
                            }
                            atomicAdd(p.bias_grad + c0 + lane, sum);
                        }
                        __syncwarp();
                    }
                }
                continue;
            }
            if (!valid) continue;
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
                    p.Z[e] = __float2bfloat16(z);
                    const __nv_bfloat16 h = __float2bfloat16(gelu(z));
                    p.H[e] = h;
                    if (p.HT) p.HT[size_t(n) * p.rows_ht + m] = h;
                    if (p.head_w) head += __bfloat162float(h) * p.head_w[n];
                } else {
                    const __nv_bfloat16 g = __float2bfloat16(acc * gelu_grad(__bfloat162float(p.zprev[e])));
                    p.H[e] = g;
                    if (p.HT) p.HT[size_t(n) * p.rows_ht + m] = g;
                    if (p.bias_grad) atomicAdd(p.bias_grad + n, __bfloat162float(g));
                }
            }
        }
        if (EPI == kForward && p.head_w) head_part[half * 128 + quarter * 32 + lane] = head;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (EPI == kForward && p.head_w && !aborted && steps > 0 && warp < 4) {
        const int r = warp * 32 + lane, m = row0 + r;
        if (m < p.rows_a) p.head_y[m] = head_part[r] + head_part[128 + r] + p.head_b[0];
    }
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(columns) : "memory");
}

}  // namespace umma
}  // namespace monki
