// Learned detector importance: a BF16 multilayer perceptron trained and evaluated on the
// GB300 by the tcgen05 GEMM of umma.cuh, with the small elementwise kernels around it.
//
// Network: F <= 64 input features (zero-padded to 64) -> 256 -> 256 -> 256 -> 1, GELU
// after each hidden layer, BF16 weights and activations, FP32 accumulation, FP32 master
// weights updated by Adam. Loss: weighted mean squared error. All row-major.
//
// Parameter vector (FP32), the layout of monki_mlp_get_params / set_params:
//   W1[256 x 64], b1[256], W2[256 x 256], b2[256], W3[256 x 256], b3[256], w4[256], b4[1]
//
// Per layer l with input X (rows x K) and weights W (256 x K):
//   forward   Z = X W^T + b (tcgen05, epilogue adds b, writes Z in BF16, H = GELU(Z), H^T;
//             the last layer's epilogue also forms the output y = H3 w4 + b4)
//   backward  dW += dZ^T X (tcgen05 split-K over the rows, A = dZ^T, B = X^T)
//             dX' = (dZ W) * GELU'(Z_prev) (tcgen05, B = W^T, epilogue applies GELU' and
//             adds the column sums of dX' to the previous layer's bias gradient)
// so every operand is K-major and the transposed activations come from the epilogues.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>

#include <cuda.h>
#include <string>
#include <vector>

#include "physics.cuh"
#include "umma.cuh"

namespace monki {
namespace mlp {

constexpr int kIn = 64;       // padded input width
constexpr int kHidden = 256;
constexpr size_t kW1 = size_t(kHidden) * kIn, kW2 = size_t(kHidden) * kHidden;
constexpr size_t kParams = kW1 + kHidden + 2 * (kW2 + kHidden) + kHidden + 1;
// Offsets into the parameter vector.
constexpr size_t oW1 = 0, ob1 = kW1, oW2 = ob1 + kHidden, ob2 = oW2 + kW2, oW3 = ob2 + kHidden, ob3 = oW3 + kW2,
                 ow4 = ob3 + kHidden, ob4 = ow4 + kHidden;

using bf16 = __nv_bfloat16;

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void write_error(char* err, size_t n, const std::string& msg) {
    if (err && n) std::snprintf(err, n, "%s", msg.c_str());
}

// ----------------------------------------------------------------------------------
// Elementwise kernels.
// ----------------------------------------------------------------------------------

// Rows of FP32 features (gathered through idx when given) into the padded BF16 input and
// its transpose; rows >= n and columns >= F are zero. Block: 256 threads over 64 rows; the
// rows are read and X written row by row, then the tile is transposed in shared memory so
// the XT rows are written as contiguous 128-byte segments too.
constexpr int kPackRows = 64, kPackStride = kIn + 1;
__global__ void __launch_bounds__(256)
pack_input(const float* __restrict__ x, const uint32_t* __restrict__ idx, int n, int F, int R,
           bf16* __restrict__ X, bf16* __restrict__ XT) {
    __shared__ bf16 tile[kPackRows * kPackStride];
    const int m0 = blockIdx.x * kPackRows;
    for (int e = threadIdx.x; e < kPackRows * kIn; e += blockDim.x) {
        const int q = e / kIn, c = e % kIn, m = m0 + q;
        float v = 0.f;
        if (m < n && c < F) v = x[size_t(idx ? idx[m] : uint32_t(m)) * F + c];
        const bf16 b = __float2bfloat16(v);
        tile[q * kPackStride + c] = b;
        if (m < R) X[size_t(m) * kIn + c] = b;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kPackRows * kIn; e += blockDim.x) {
        const int c = e / kPackRows, q = e % kPackRows, m = m0 + q;
        if (m < R) XT[size_t(c) * R + m] = tile[q * kPackStride + c];
    }
}

__global__ void gather_targets(const float* __restrict__ t, const float* __restrict__ w, const uint32_t* __restrict__ idx,
                               int n, int R, float* __restrict__ tb, float* __restrict__ wb) {
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < R; m += gridDim.x * blockDim.x) {
        tb[m] = m < n ? t[idx ? idx[m] : uint32_t(m)] : 0.f;
        wb[m] = m < n ? w[idx ? idx[m] : uint32_t(m)] : 0.f;
    }
}

// Minibatch indices: Philox4x32-10 counter (step, i / 4, 1, 0), key (seed, 0).
__global__ void sample_indices(uint32_t step, uint32_t seed, int batch, uint32_t n, uint32_t* __restrict__ idx) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < batch; i += gridDim.x * blockDim.x) {
        const uint4 w = philox4x32_10(make_uint4(step, uint32_t(i) >> 2, 1u, 0u), make_uint2(seed, 0u));
        const uint32_t lane = uint32_t(i) & 3u;
        const uint32_t r = lane == 0 ? w.x : lane == 1 ? w.y : lane == 2 ? w.z : w.w;
        idx[i] = uint32_t((uint64_t(r) * n) >> 32);
    }
}

// dy = 2 w (y - t) / sum(w); loss accumulates sum w (y - t)^2 / sum(w).
__global__ void loss_grad(const float* __restrict__ y, const float* __restrict__ t, const float* __restrict__ w,
                          int rows, float inv_weight, float* __restrict__ dy, float* __restrict__ loss) {
    float part = 0.f;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < rows; m += gridDim.x * blockDim.x) {
        const float d = y[m] - t[m];
        dy[m] = 2.f * w[m] * d * inv_weight;
        part += w[m] * d * d * inv_weight;
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) part += __shfl_xor_sync(0xffffffffu, part, off);
    if ((threadIdx.x & 31) == 0 && part != 0.f) atomicAdd(loss, part);
}

// Output layer backward: dw4 += dy^T H3, db4 += sum dy, dZ3 = dy w4^T * GELU'(Z3) in BF16,
// its transpose and db3 += the column sums of dZ3. Block: 256 threads (one per hidden unit)
// over a slab of 64 rows; the slab's dZ3 is staged in shared memory (odd row stride, so the
// column reads are free of bank conflicts) and each warp then writes 32 rows of the
// transpose as 128-byte segments. Rows from `rows` to the slab's end are written as zeros.
constexpr int kSlab = 64, kSlabStride = kHidden + 1;
__global__ void __launch_bounds__(kHidden)
head_backward(const float* __restrict__ dy, const bf16* __restrict__ H, const float* __restrict__ w4,
              const bf16* __restrict__ Z, int rows, int R, float* __restrict__ grads, bf16* __restrict__ G,
              bf16* __restrict__ GT) {
    __shared__ bf16 tile[kSlab * kSlabStride];
    const int n = threadIdx.x;
    const int m0 = blockIdx.x * kSlab;
    float acc = 0.f, bias = 0.f, column = 0.f;
    const float wn = w4[n];
    // Eight rows in flight per thread: their loads are issued before any is used (rows past
    // `rows` are inside the R-row buffers, read and then masked).
    for (int q0 = 0; q0 < kSlab; q0 += 8) {
        float d[8];
        bf16 h[8], z[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int m = m0 + q0 + u;
            const size_t at = size_t(m) * kHidden + n;
            d[u] = m < rows ? dy[m] : 0.f;
            h[u] = H[at];
            z[u] = Z[at];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int m = m0 + q0 + u;
            bf16 g = __float2bfloat16(0.f);
            if (m < rows) {
                acc += d[u] * __bfloat162float(h[u]);
                bias += d[u];
                g = __float2bfloat16(d[u] * wn * umma::gelu_grad(__bfloat162float(z[u])));
                G[size_t(m) * kHidden + n] = g;
                column += __bfloat162float(g);
            }
            tile[(q0 + u) * kSlabStride + n] = g;
        }
    }
    atomicAdd(grads + ow4 + n, acc);
    atomicAdd(grads + ob3 + n, column);
    if (n == 0) atomicAdd(grads + ob4, bias);
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m = m0 + 2 * lane;
    for (int c = warp; c < kHidden; c += kHidden / 32) {
        __nv_bfloat162 pair;
        pair.x = tile[(2 * lane) * kSlabStride + c];
        pair.y = tile[(2 * lane + 1) * kSlabStride + c];
        bf16* dst = GT + size_t(c) * R + m;
        if (m + 1 < R) *reinterpret_cast<__nv_bfloat162*>(dst) = pair;
        else if (m < R) dst[0] = pair.x;
    }
}

__global__ void adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                     size_t count, float lr, float c1, float c2) {
    for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < count; e += size_t(gridDim.x) * blockDim.x) {
        const float gi = g[e];
        const float a = 0.9f * m1[e] + 0.1f * gi;
        const float b = 0.999f * m2[e] + 0.001f * gi * gi;
        m1[e] = a;
        m2[e] = b;
        p[e] -= lr * (a * c1) / (sqrtf(b * c2) + 1e-8f);
    }
}

// BF16 working copies of the weights and the transposes the backward pass needs.
__global__ void refresh(const float* __restrict__ p, bf16* __restrict__ W1, bf16* __restrict__ W2, bf16* __restrict__ W3,
                        bf16* __restrict__ W2T, bf16* __restrict__ W3T) {
    for (size_t e = blockIdx.x * size_t(blockDim.x) + threadIdx.x; e < kW2; e += size_t(gridDim.x) * blockDim.x) {
        const size_t r = e / kHidden, c = e % kHidden;
        if (e < kW1) W1[e] = __float2bfloat16(p[oW1 + e]);
        const bf16 w2 = __float2bfloat16(p[oW2 + e]), w3 = __float2bfloat16(p[oW3 + e]);
        W2[e] = w2;
        W3[e] = w3;
        W2T[c * kHidden + r] = w2;
        W3T[c * kHidden + r] = w3;
    }
}

// ----------------------------------------------------------------------------------
// Session.
// ----------------------------------------------------------------------------------
struct Net {
    int device = 0, features = 0, R = 0;  // R: rows per pass, a multiple of 128
    cudaStream_t stream = nullptr;
    float *params = nullptr, *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
    bf16 *W1 = nullptr, *W2 = nullptr, *W3 = nullptr, *W2T = nullptr, *W3T = nullptr;
    bf16 *X = nullptr, *XT = nullptr, *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *H1T = nullptr, *H2T = nullptr;
    bf16 *G3 = nullptr, *G3T = nullptr, *G2 = nullptr, *G2T = nullptr, *G1 = nullptr, *G1T = nullptr;
    bf16 *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr;  // pre-activations
    float *y = nullptr, *dy = nullptr, *tb = nullptr, *wb = nullptr;
    float* loss = nullptr;
    uint32_t* failure = nullptr;
    uint32_t* idx = nullptr;
    float *data_x = nullptr, *data_t = nullptr, *data_w = nullptr;
    uint32_t data_n = 0;
    uint32_t step = 0, seed = 0;
    std::vector<void*> owned;

    template <typename P>
    P* alloc(size_t count) {
        void* p = nullptr;
        check(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(P)), "cudaMalloc");
        owned.push_back(p);
        return static_cast<P*>(p);
    }
    ~Net() {
        if (stream) cudaStreamSynchronize(stream);
        for (void* p : owned) cudaFree(p);
        cudaFree(data_x); cudaFree(data_t); cudaFree(data_w);
        if (stream) cudaStreamDestroy(stream);
    }
};

std::mutex g_attr_lock;
bool g_attr_done[64] = {};

void configure(int device) {
    std::lock_guard<std::mutex> guard(g_attr_lock);
    if (device < 0 || device >= 64 || g_attr_done[device]) return;
    check(cudaFuncSetAttribute(umma::gemm<umma::kStore>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma::kSmemBytes), "attr");
    check(cudaFuncSetAttribute(umma::gemm<umma::kForward>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma::kSmemBytes), "attr");
    check(cudaFuncSetAttribute(umma::gemm<umma::kBackward>, cudaFuncAttributeMaxDynamicSharedMemorySize, umma::kSmemBytes), "attr");
    check(cudaFuncSetAttribute(umma::gemm<umma::kAccumulate>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               umma::smem_bytes_of<umma::kAccumulate>()), "attr");
    g_attr_done[device] = true;
}

// cuTensorMapEncodeTiled, from the driver through the runtime (no link against libcuda).
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult found{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &found) == cudaSuccess &&
            found == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(f);
    });
    if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is unavailable from the driver");
    return fn;
}

// Tensor map of a K-major BF16 matrix (rows x k_extent, row stride ld elements) read in
// tiles of 64 K-elements (128 bytes, the swizzle width) x box_rows rows; reads outside the
// matrix return zeros.
CUtensorMap tile_map(const bf16* base, int rows, int k_extent, int ld, int box_rows) {
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (size_t(ld) * sizeof(bf16)) % 16 || k_extent % umma::kBlockK ||
        box_rows < 1 || box_rows > 256)
        throw std::runtime_error("operand outside the tensor-map tiling");
    CUtensorMap map{};
    const cuuint64_t dims[2] = {cuuint64_t(k_extent), cuuint64_t(rows)};
    const cuuint64_t strides[1] = {cuuint64_t(ld) * sizeof(bf16)};
    const cuuint32_t box[2] = {cuuint32_t(umma::kBlockK), cuuint32_t(box_rows)};
    const cuuint32_t element[2] = {1, 1};
    const CUresult r = encoder()(&map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(base), dims, strides, box,
                                 element, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed (" + std::to_string(int(r)) + ")");
    return map;
}

// One GEMM: operands (K-major, row strides lda / ldb) and the epilogue's parameters.
struct Gemm {
    const bf16* A;
    int lda;
    const bf16* B;
    int ldb;
    umma::Params p;
};

template <int EPI>
void gemm(const Gemm& g, int splits, cudaStream_t stream) {
    const umma::Params& p = g.p;
    if (p.K % umma::kBlockK || p.k_chunk % umma::kBlockK || p.N % 16 || p.N < 16 || p.N > 256 || p.rows_a < 1)
        throw std::runtime_error("GEMM shape outside the kernel's tiling");
    const CUtensorMap map_a = tile_map(g.A, p.rows_a, p.K, g.lda, umma::kBlockM);
    const CUtensorMap map_b = tile_map(g.B, p.N, p.K, g.ldb, p.N);
    dim3 grid((p.rows_a + umma::kBlockM - 1) / umma::kBlockM, splits);
    umma::gemm<EPI><<<grid, umma::kThreads, umma::smem_bytes_of<EPI>(), stream>>>(map_a, map_b, p);
    check(cudaGetLastError(), "gemm launch");
}

Gemm params_for(const bf16* A, const bf16* B, int rows, int N, int K, uint32_t* failure) {
    Gemm g{A, K, B, K, umma::Params{}};
    g.p.rows_a = rows; g.p.N = N; g.p.K = K; g.p.k_chunk = K;
    g.p.failure = failure;
    return g;
}

// Zero the columns [rows, rows rounded up to 64) of a transposed (height x R) matrix: the
// split-K weight-gradient GEMMs read whole 64-column slices.
void clear_tail(bf16* T, int rows, int R, int height, cudaStream_t stream) {
    const int end = std::min(R, (rows + 63) / 64 * 64);
    if (end > rows)
        check(cudaMemset2DAsync(T + rows, size_t(R) * sizeof(bf16), 0, size_t(end - rows) * sizeof(bf16), size_t(height), stream),
              "memset(tail)");
}

// Forward pass of the first `rows` rows (<= R) of the packed input.
void forward(Net& n, int rows) {
    const int R = n.R;
    Gemm g = params_for(n.X, n.W1, rows, kHidden, kIn, n.failure);
    g.p.Z = n.Z1; g.p.bias = n.params + ob1; g.p.H = n.H1; g.p.HT = n.H1T; g.p.rows_ht = R;
    gemm<umma::kForward>(g, 1, n.stream);
    g = params_for(n.H1, n.W2, rows, kHidden, kHidden, n.failure);
    g.p.Z = n.Z2; g.p.bias = n.params + ob2; g.p.H = n.H2; g.p.HT = n.H2T; g.p.rows_ht = R;
    gemm<umma::kForward>(g, 1, n.stream);
    g = params_for(n.H2, n.W3, rows, kHidden, kHidden, n.failure);
    g.p.Z = n.Z3; g.p.bias = n.params + ob3; g.p.H = n.H3; g.p.HT = nullptr; g.p.rows_ht = R;
    // The output layer rides on this epilogue: y = H3 w4 + b4.
    g.p.head_w = n.params + ow4; g.p.head_b = n.params + ob4; g.p.head_y = n.y;
    gemm<umma::kForward>(g, 1, n.stream);
    clear_tail(n.H1T, rows, R, kHidden, n.stream);
    clear_tail(n.H2T, rows, R, kHidden, n.stream);
}

// Loss and gradients of the first `rows` rows against tb / wb (gradients accumulate into
// n.grads, which the caller clears).
void backward(Net& n, int rows, float inv_weight, float* loss) {
    const int R = n.R;
    loss_grad<<<256, 256, 0, n.stream>>>(n.y, n.tb, n.wb, rows, inv_weight, n.dy, loss);
    head_backward<<<(rows + 63) / 64, kHidden, 0, n.stream>>>(n.dy, n.H3, n.params + ow4, n.Z3, rows, R, n.grads,
                                                              n.G3, n.G3T);
    check(cudaGetLastError(), "head backward launch");
    // Split-K over the rows for the weight gradients: 64-row multiples, slices of 1,024 rows
    // (at batch 65,536 two row tiles x 64 slices = 128 CTAs, each adding one partial).
    const int chunk = 1024, K = (rows + 63) / 64 * 64, splits = (K + chunk - 1) / chunk;
    Gemm g = params_for(n.G3T, n.H2T, kHidden, kHidden, K, n.failure);
    g.lda = R; g.ldb = R; g.p.k_chunk = chunk; g.p.C = n.grads + oW3;
    gemm<umma::kAccumulate>(g, splits, n.stream);
    g = params_for(n.G3, n.W3T, rows, kHidden, kHidden, n.failure);
    g.p.zprev = n.Z2; g.p.H = n.G2; g.p.HT = n.G2T; g.p.rows_ht = R; g.p.bias_grad = n.grads + ob2;
    gemm<umma::kBackward>(g, 1, n.stream);
    clear_tail(n.G2T, rows, R, kHidden, n.stream);
    g = params_for(n.G2T, n.H1T, kHidden, kHidden, K, n.failure);
    g.lda = R; g.ldb = R; g.p.k_chunk = chunk; g.p.C = n.grads + oW2;
    gemm<umma::kAccumulate>(g, splits, n.stream);
    g = params_for(n.G2, n.W2T, rows, kHidden, kHidden, n.failure);
    g.p.zprev = n.Z1; g.p.H = n.G1; g.p.HT = n.G1T; g.p.rows_ht = R; g.p.bias_grad = n.grads + ob1;
    gemm<umma::kBackward>(g, 1, n.stream);
    clear_tail(n.G1T, rows, R, kHidden, n.stream);
    g = params_for(n.G1T, n.XT, kHidden, kIn, K, n.failure);
    g.lda = R; g.ldb = R; g.p.k_chunk = chunk; g.p.C = n.grads + oW1;
    gemm<umma::kAccumulate>(g, splits, n.stream);
    check(cudaGetLastError(), "backward launch");
}

void refresh_weights(Net& n) {
    refresh<<<256, 256, 0, n.stream>>>(n.params, n.W1, n.W2, n.W3, n.W2T, n.W3T);
    check(cudaGetLastError(), "refresh launch");
}

void check_failure(Net& n) {
    uint32_t flag = 0;
    check(cudaMemcpyAsync(&flag, n.failure, sizeof(flag), cudaMemcpyDeviceToHost, n.stream), "copy(failure)");
    check(cudaStreamSynchronize(n.stream), "mlp");
    if (flag) throw std::runtime_error("tensor-core GEMM wait gave up (flag " + std::to_string(flag) + ")");
}

}  // namespace mlp
}  // namespace monki

using monki::mlp::Net;
using namespace monki::mlp;
namespace umma = monki::umma;

extern "C" {

size_t monki_mlp_param_count(void) { return kParams; }

void* monki_mlp_create(uint32_t device, uint32_t features, uint32_t rows, uint32_t seed, char* err, size_t errlen) {
    Net* n = nullptr;
    try {
        if (features < 1 || features > uint32_t(kIn)) throw std::runtime_error("features must be in [1, 64]");
        if (rows < 1 || rows > (1u << 20)) throw std::runtime_error("rows must be in [1, 2^20]");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || device >= uint32_t(count))
            throw std::runtime_error("Requested CUDA device is unavailable");
        check(cudaSetDevice(int(device)), "cudaSetDevice");
        cudaDeviceProp prop{};
        check(cudaGetDeviceProperties(&prop, int(device)), "cudaGetDeviceProperties");
        if (prop.major != 10 || prop.minor != 3) throw std::runtime_error("The learned importance kernels need an sm_103 GPU");
        configure(int(device));
        n = new Net();
        n->device = int(device);
        n->features = int(features);
        n->R = int((rows + 127) / 128 * 128);
        n->seed = seed;
        check(cudaStreamCreateWithFlags(&n->stream, cudaStreamNonBlocking), "stream");
        const size_t R = size_t(n->R), H = size_t(kHidden);
        n->params = n->alloc<float>(kParams); n->grads = n->alloc<float>(kParams);
        n->m1 = n->alloc<float>(kParams); n->m2 = n->alloc<float>(kParams);
        n->W1 = n->alloc<bf16>(kW1); n->W2 = n->alloc<bf16>(kW2); n->W3 = n->alloc<bf16>(kW2);
        n->W2T = n->alloc<bf16>(kW2); n->W3T = n->alloc<bf16>(kW2);
        n->X = n->alloc<bf16>(R * kIn); n->XT = n->alloc<bf16>(R * kIn);
        for (bf16** b : {&n->H1, &n->H2, &n->H3, &n->H1T, &n->H2T, &n->G3, &n->G3T, &n->G2, &n->G2T, &n->G1, &n->G1T})
            *b = n->alloc<bf16>(R * H);
        n->Z1 = n->alloc<bf16>(R * H); n->Z2 = n->alloc<bf16>(R * H); n->Z3 = n->alloc<bf16>(R * H);
        n->y = n->alloc<float>(R); n->dy = n->alloc<float>(R); n->tb = n->alloc<float>(R); n->wb = n->alloc<float>(R);
        n->loss = n->alloc<float>(1);
        n->failure = n->alloc<uint32_t>(1);
        n->idx = n->alloc<uint32_t>(R);
        check(cudaMemset(n->params, 0, kParams * sizeof(float)), "memset");
        check(cudaMemset(n->m1, 0, kParams * sizeof(float)), "memset");
        check(cudaMemset(n->m2, 0, kParams * sizeof(float)), "memset");
        check(cudaMemset(n->failure, 0, sizeof(uint32_t)), "memset");
        // Transposed activations are read in 64-row slices; the padding rows stay zero.
        for (bf16* b : {n->XT, n->H1T, n->H2T, n->G3T, n->G2T, n->G1T})
            check(cudaMemset(b, 0, R * (b == n->XT ? size_t(kIn) : H) * sizeof(bf16)), "memset");
        refresh_weights(*n);
        check(cudaStreamSynchronize(n->stream), "create");
        return n;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        delete n;
        return nullptr;
    }
}

int monki_mlp_set_params(void* handle, const float* params, size_t count, char* err, size_t errlen) {
    Net* n = static_cast<Net*>(handle);
    try {
        if (!n || !params || count != kParams) throw std::runtime_error("set_params needs the full parameter vector");
        for (size_t e = 0; e < count; ++e)
            if (!std::isfinite(params[e])) throw std::runtime_error("Nonfinite parameter");
        check(cudaSetDevice(n->device), "cudaSetDevice");
        check(cudaMemcpyAsync(n->params, params, kParams * sizeof(float), cudaMemcpyHostToDevice, n->stream), "upload");
        check(cudaMemsetAsync(n->m1, 0, kParams * sizeof(float), n->stream), "memset");
        check(cudaMemsetAsync(n->m2, 0, kParams * sizeof(float), n->stream), "memset");
        n->step = 0;
        refresh_weights(*n);
        check(cudaStreamSynchronize(n->stream), "set_params");
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_mlp_get_params(void* handle, float* params, size_t count, char* err, size_t errlen) {
    Net* n = static_cast<Net*>(handle);
    try {
        if (!n || !params || count != kParams) throw std::runtime_error("get_params needs the full parameter vector");
        check(cudaSetDevice(n->device), "cudaSetDevice");
        check(cudaMemcpyAsync(params, n->params, kParams * sizeof(float), cudaMemcpyDeviceToHost, n->stream), "download");
        check(cudaStreamSynchronize(n->stream), "get_params");
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

// y[rows] = network(x[rows x features]), any number of rows (processed R at a time).
int monki_mlp_forward(void* handle, const float* x, uint32_t rows, float* y, char* err, size_t errlen) {
    Net* n = static_cast<Net*>(handle);
    try {
        if (!n || (!x && rows) || (!y && rows)) throw std::runtime_error("Invalid network or buffers");
        check(cudaSetDevice(n->device), "cudaSetDevice");
        float* dx = nullptr;
        check(cudaMalloc(&dx, std::max<size_t>(1, size_t(std::min<uint32_t>(rows, uint32_t(n->R))) * n->features * sizeof(float))), "cudaMalloc");
        try {
            for (uint32_t r0 = 0; r0 < rows; r0 += uint32_t(n->R)) {
                const int m = int(std::min<uint32_t>(uint32_t(n->R), rows - r0));
                check(cudaMemcpyAsync(dx, x + size_t(r0) * n->features, size_t(m) * n->features * sizeof(float),
                                      cudaMemcpyHostToDevice, n->stream), "upload");
                pack_input<<<(n->R + kPackRows - 1) / kPackRows, 256, 0, n->stream>>>(dx, nullptr, m, n->features, n->R, n->X, n->XT);
                forward(*n, m);
                check(cudaMemcpyAsync(y + r0, n->y, size_t(m) * sizeof(float), cudaMemcpyDeviceToHost, n->stream), "download");
                check_failure(*n);
            }
        } catch (...) {
            cudaFree(dx);
            throw;
        }
        cudaFree(dx);
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

// Loss and gradient (the parameter vector's layout) of one batch of rows <= R.
int monki_mlp_gradients(void* handle, const float* x, const float* target, const float* weight, uint32_t rows,
                        float* grads, float* loss, char* err, size_t errlen) {
    Net* n = static_cast<Net*>(handle);
    try {
        if (!n || !x || !target || !weight || !grads || !loss || rows < 1 || rows > uint32_t(n->R))
            throw std::runtime_error("Invalid network, buffers or row count");
        double total = 0.0;
        for (uint32_t m = 0; m < rows; ++m) total += weight[m];
        if (!(total > 0.0)) throw std::runtime_error("Weights must have a positive sum");
        check(cudaSetDevice(n->device), "cudaSetDevice");
        float *dx = nullptr, *dt = nullptr, *dw = nullptr;
        check(cudaMalloc(&dx, size_t(rows) * n->features * sizeof(float)), "cudaMalloc");
        check(cudaMalloc(&dt, rows * sizeof(float)), "cudaMalloc");
        check(cudaMalloc(&dw, rows * sizeof(float)), "cudaMalloc");
        check(cudaMemcpyAsync(dx, x, size_t(rows) * n->features * sizeof(float), cudaMemcpyHostToDevice, n->stream), "upload");
        check(cudaMemcpyAsync(dt, target, rows * sizeof(float), cudaMemcpyHostToDevice, n->stream), "upload");
        check(cudaMemcpyAsync(dw, weight, rows * sizeof(float), cudaMemcpyHostToDevice, n->stream), "upload");
        pack_input<<<(n->R + kPackRows - 1) / kPackRows, 256, 0, n->stream>>>(dx, nullptr, int(rows), n->features, n->R, n->X, n->XT);
        gather_targets<<<256, 256, 0, n->stream>>>(dt, dw, nullptr, int(rows), n->R, n->tb, n->wb);
        check(cudaMemsetAsync(n->grads, 0, kParams * sizeof(float), n->stream), "memset");
        check(cudaMemsetAsync(n->loss, 0, sizeof(float), n->stream), "memset");
        forward(*n, int(rows));
        backward(*n, int(rows), float(1.0 / total), n->loss);
        check(cudaMemcpyAsync(grads, n->grads, kParams * sizeof(float), cudaMemcpyDeviceToHost, n->stream), "download");
        check(cudaMemcpyAsync(loss, n->loss, sizeof(float), cudaMemcpyDeviceToHost, n->stream), "download");
        check_failure(*n);
        cudaFree(dx); cudaFree(dt); cudaFree(dw);
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

// Keep a training set on the device: rows x features inputs, targets and weights.
int monki_mlp_set_data(void* handle, const float* x, const float* target, const float* weight, uint32_t rows,
                       char* err, size_t errlen) {
    Net* n = static_cast<Net*>(handle);
    try {
        if (!n || !x || !target || !weight || rows < 1) throw std::runtime_error("Invalid network or training set");
        check(cudaSetDevice(n->device), "cudaSetDevice");
        check(cudaStreamSynchronize(n->stream), "sync");
        cudaFree(n->data_x); cudaFree(n->data_t); cudaFree(n->data_w);
        n->data_x = n->data_t = n->data_w = nullptr;
        n->data_n = 0;
        check(cudaMalloc(&n->data_x, size_t(rows) * n->features * sizeof(float)), "cudaMalloc");
        check(cudaMalloc(&n->data_t, rows * sizeof(float)), "cudaMalloc");
        check(cudaMalloc(&n->data_w, rows * sizeof(float)), "cudaMalloc");
        check(cudaMemcpy(n->data_x, x, size_t(rows) * n->features * sizeof(float), cudaMemcpyHostToDevice), "upload");
        check(cudaMemcpy(n->data_t, target, rows * sizeof(float), cudaMemcpyHostToDevice), "upload");
        check(cudaMemcpy(n->data_w, weight, rows * sizeof(float), cudaMemcpyHostToDevice), "upload");
        n->data_n = rows;
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

// Adam steps on minibatches of `batch` rows (<= R) drawn with replacement from the
// device training set; losses[steps] receives each step's minibatch loss.
int monki_mlp_train(void* handle, uint32_t steps, uint32_t batch, float lr, float* losses, char* err, size_t errlen) {
    Net* n = static_cast<Net*>(handle);
    try {
        if (!n || !n->data_n) throw std::runtime_error("No training set on the device");
        if (batch < 1 || batch > uint32_t(n->R)) throw std::runtime_error("batch must be in [1, rows of the network]");
        if (!(lr > 0.f) || !std::isfinite(lr)) throw std::runtime_error("Invalid learning rate");
        check(cudaSetDevice(n->device), "cudaSetDevice");
        std::vector<float> host_loss(steps, 0.f);
        float* dloss = nullptr;
        check(cudaMalloc(&dloss, std::max<size_t>(steps, 1) * sizeof(float)), "cudaMalloc");
        try {
            check(cudaMemsetAsync(dloss, 0, std::max<size_t>(steps, 1) * sizeof(float), n->stream), "memset");
            for (uint32_t s = 0; s < steps; ++s) {
                const uint32_t t = ++n->step;
                sample_indices<<<(batch + 255) / 256, 256, 0, n->stream>>>(t, n->seed, int(batch), n->data_n, n->idx);
                pack_input<<<(n->R + kPackRows - 1) / kPackRows, 256, 0, n->stream>>>(n->data_x, n->idx, int(batch), n->features, n->R, n->X, n->XT);
                gather_targets<<<256, 256, 0, n->stream>>>(n->data_t, n->data_w, n->idx, int(batch), n->R, n->tb, n->wb);
                check(cudaMemsetAsync(n->grads, 0, kParams * sizeof(float), n->stream), "memset");
                forward(*n, int(batch));
                // Weighted mean over the minibatch: normalised by the batch size (the
                // targets' weights average to about one), so the gradient scale does not
                // depend on the batch.
                backward(*n, int(batch), 1.0f / float(batch), dloss + s);
                const float c1 = 1.f / (1.f - std::pow(0.9f, float(t))), c2 = 1.f / (1.f - std::pow(0.999f, float(t)));
                adam<<<592, 256, 0, n->stream>>>(n->params, n->grads, n->m1, n->m2, kParams, lr, c1, c2);
                refresh_weights(*n);
                check(cudaGetLastError(), "train launch");
            }
            check(cudaMemcpyAsync(host_loss.data(), dloss, steps * sizeof(float), cudaMemcpyDeviceToHost, n->stream), "download");
            check_failure(*n);
        } catch (...) {
            cudaFree(dloss);
            throw;
        }
        cudaFree(dloss);
        if (losses) std::copy(host_loss.begin(), host_loss.end(), losses);
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

void monki_mlp_close(void* handle) {
    Net* n = static_cast<Net*>(handle);
    if (!n) return;
    cudaSetDevice(n->device);
    delete n;
}

// Test hook: C (M x N, FP32) = A (M x K) B^T (N x K), BF16 bits in, through the tcgen05
// GEMM; splits > 1 runs split-K into a zeroed C with the accumulating epilogue.
int monki_mlp_gemm_probe(uint32_t device, const uint16_t* a, const uint16_t* b, int M, int N, int K, int splits,
                         float* c, char* err, size_t errlen) {
    try {
        if (!a || !b || !c || M < 1 || splits < 1 || K % 64 || N % 16 || N < 16 || N > 256 || (K / 64) % splits)
            throw std::runtime_error("Invalid GEMM probe shape");
        check(cudaSetDevice(int(device)), "cudaSetDevice");
        configure(int(device));
        bf16 *da = nullptr, *db = nullptr;
        float* dc = nullptr;
        uint32_t* flag = nullptr;
        check(cudaMalloc(&da, size_t(M) * K * 2), "cudaMalloc");
        check(cudaMalloc(&db, size_t(N) * K * 2), "cudaMalloc");
        check(cudaMalloc(&dc, size_t(M) * N * 4), "cudaMalloc");
        check(cudaMalloc(&flag, 4), "cudaMalloc");
        check(cudaMemcpy(da, a, size_t(M) * K * 2, cudaMemcpyHostToDevice), "upload");
        check(cudaMemcpy(db, b, size_t(N) * K * 2, cudaMemcpyHostToDevice), "upload");
        check(cudaMemset(dc, 0, size_t(M) * N * 4), "memset");
        check(cudaMemset(flag, 0, 4), "memset");
        Gemm g = params_for(da, db, M, N, K, flag);
        g.p.C = dc;
        g.p.k_chunk = K / splits;
        if (splits == 1) gemm<umma::kStore>(g, 1, nullptr);
        else gemm<umma::kAccumulate>(g, splits, nullptr);
        uint32_t f = 0;
        check(cudaMemcpy(&f, flag, 4, cudaMemcpyDeviceToHost), "download");
        check(cudaMemcpy(c, dc, size_t(M) * N * 4, cudaMemcpyDeviceToHost), "download");
        cudaFree(da); cudaFree(db); cudaFree(dc); cudaFree(flag);
        if (f) throw std::runtime_error("tensor-core GEMM wait gave up");
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

}  // extern "C"
