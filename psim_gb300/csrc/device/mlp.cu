// The warm-start surrogate's multilayer perceptron: BF16 parameters and activations, FP32
// accumulation, GELU hidden layers, a linear output, mean-squared-error loss and Adam with FP32
// master weights.  Everything runs in a handful of hand-written kernels:
//   gemm_kernel      C = op(A) op(B) on the tensor cores (mma.sync m16n8k16, BF16 operands staged
//                    in shared memory, FP32 sums)
//   bias_act_kernel  Z = C + b, and the BF16 activation GELU(Z) (hidden) or Z (output)
//   mse_kernel       dY = 2 (Y - T) / (n outputs), and the loss
//   gelu_bwd_kernel  dZ = dA GELU'(Z)
//   bias_grad_kernel db = column sums of dZ
//   adam_kernel      Adam update of the master weights and their BF16 copy
// The network is small (about 0.5 M parameters): a step is a few microseconds of GPU time.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include <algorithm>
#include <cmath>
#include <numeric>
#include <random>
#include <stdexcept>
#include <string>
#include <vector>

#include "mlp.hpp"

namespace psim::gpu {

namespace {

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) { throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e)); }
}

template<typename T> struct DevArray {
    T* p{ nullptr };
    std::size_t n{ 0 };
    DevArray() = default;
    explicit DevArray(std::size_t count) { resize(count); }
    ~DevArray() {
        if (p != nullptr) { cudaFree(p); }
    }
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    DevArray(DevArray&& o) noexcept : p{ o.p }, n{ o.n } {
        o.p = nullptr;
        o.n = 0;
    }
    DevArray& operator=(DevArray&& o) noexcept {
        std::swap(p, o.p);
        std::swap(n, o.n);
        return *this;
    }
    void resize(std::size_t count) {
        if (count <= n && p != nullptr) { return; }
        if (p != nullptr) { cudaFree(p); }
        p = nullptr;
        n = 0;
        check(cudaMalloc(&p, std::max<std::size_t>(count, 1) * sizeof(T)), "cudaMalloc");
        n = count;
    }
};

// GEMM tiles: a 64 x 64 block of C per 128-thread block (four warps of 32 x 32), K in steps of
// 16.  Operand tiles are staged in shared memory as BF16 with k contiguous, zero-padded at the
// matrix edges, and multiplied on the tensor cores by mma.sync m16n8k16 (BF16 in, FP32 sums).
constexpr int kBM = 64;
constexpr int kBN = 64;
constexpr int kBK = 16;
constexpr int kPadK = kBK + 8;// row pitch in elements: 48 bytes, so the fragment loads of a warp spread over the banks

// One m16n8k16 product: c += a (16 x 16, row-major fragment) b (16 x 8, column-major fragment).
__device__ __forceinline__ void mma_bf16_16816(float c[4], const std::uint32_t a[4], const std::uint32_t b[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// C[M][N] = op(A)[M][K] op(B)[K][N].  op(A)(m, k) = A[k*M + m] when transA else A[m*K + k];
// op(B)(k, n) = B[n*K + k] when transB else B[k*N + n].
__global__ void __launch_bounds__(128) gemm_kernel(const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M, int N, int K,
                                                   bool transA, bool transB) {
    __shared__ __align__(16) __nv_bfloat16 As[kBM][kPadK];// [m][k]
    __shared__ __align__(16) __nv_bfloat16 Bs[kBN][kPadK];// [n][k]
    const int tid = static_cast<int>(threadIdx.x);
    const int warp = tid >> 5;
    const int lane = tid & 31;
    const int group = lane >> 2;// fragment row (A, C) or column (B)
    const int tig = lane & 3;   // thread in group: fragment k pair (A, B) or column pair (C)
    const int m0 = static_cast<int>(blockIdx.y) * kBM;
    const int n0 = static_cast<int>(blockIdx.x) * kBN;
    const int wm = (warp >> 1) * 32;// the warp's 32 x 32 sub-tile
    const int wn = (warp & 1) * 32;
    const __nv_bfloat16 zero = __float2bfloat16_rn(0.f);
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int r = 0; r < 4; ++r) { acc[i][j][r] = 0.f; }
        }
    }
    for (int k0 = 0; k0 < K; k0 += kBK) {
        // stage op(A)[m0.., k0..] and op(B)[k0.., n0..] (transposed to [n][k]): 8 elements each per thread
#pragma unroll
        for (int e = 0; e < (kBM * kBK) / 128; ++e) {
            const int idx = tid + e * 128;
            const int r = idx / kBK;
            const int k = idx % kBK;
            const int m = m0 + r;
            const int kk = k0 + k;
            __nv_bfloat16 v = zero;
            if (m < M && kk < K) { v = transA ? A[static_cast<std::size_t>(kk) * M + m] : A[static_cast<std::size_t>(m) * K + kk]; }
            As[r][k] = v;
            const int n = n0 + r;
            __nv_bfloat16 w = zero;
            if (n < N && kk < K) { w = transB ? B[static_cast<std::size_t>(n) * K + kk] : B[static_cast<std::size_t>(kk) * N + n]; }
            Bs[r][k] = w;
        }
        __syncthreads();
        std::uint32_t af[2][4];
        std::uint32_t bf[4][2];
#pragma unroll
        for (int i = 0; i < 2; ++i) {// A fragments: rows group / group + 8, k pairs 2 tig / 2 tig + 8
            const int r = wm + i * 16 + group;
            af[i][0] = *reinterpret_cast<const std::uint32_t*>(&As[r][2 * tig]);
            af[i][1] = *reinterpret_cast<const std::uint32_t*>(&As[r + 8][2 * tig]);
            af[i][2] = *reinterpret_cast<const std::uint32_t*>(&As[r][2 * tig + 8]);
            af[i][3] = *reinterpret_cast<const std::uint32_t*>(&As[r + 8][2 * tig + 8]);
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {// B fragments: column group, k pairs 2 tig / 2 tig + 8
            const int c = wn + j * 8 + group;
            bf[j][0] = *reinterpret_cast<const std::uint32_t*>(&Bs[c][2 * tig]);
            bf[j][1] = *reinterpret_cast<const std::uint32_t*>(&Bs[c][2 * tig + 8]);
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
#pragma unroll
            for (int j = 0; j < 4; ++j) { mma_bf16_16816(acc[i][j], af[i], bf[j]); }
        }
        __syncthreads();
    }
    // C fragments: rows group / group + 8, columns 2 tig, 2 tig + 1
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int r = m0 + wm + i * 16 + group;
            const int c = n0 + wn + j * 8 + 2 * tig;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int rr = r + h * 8;
                if (rr >= M) { continue; }
                if (c < N) { C[static_cast<std::size_t>(rr) * N + c] = acc[i][j][2 * h]; }
                if (c + 1 < N) { C[static_cast<std::size_t>(rr) * N + c + 1] = acc[i][j][2 * h + 1]; }
            }
        }
    }
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float z) {
    return 0.5f * (1.f + erff(z * 0.70710678118654752f)) + z * expf(-0.5f * z * z) * 0.39894228040143268f;
}

// Z = C + b over [M][N]; hidden layers store Z and the BF16 activation, the output layer Z only.
__global__ void bias_act_kernel(const float* C, const float* b, float* Z, __nv_bfloat16* act, int M, int N, bool hidden) {
    const std::size_t total = static_cast<std::size_t>(M) * N;
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x) {
        const float z = C[i] + b[i % N];
        Z[i] = z;
        if (hidden) { act[i] = __float2bfloat16_rn(gelu(z)); }
    }
}

__global__ void mse_kernel(const float* Y, const float* T, __nv_bfloat16* dY, std::size_t total, float scale, float* loss) {
    float part = 0.f;
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x) {
        const float d = Y[i] - T[i];
        part += d * d;
        dY[i] = __float2bfloat16_rn(2.f * d * scale);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) { part += __shfl_down_sync(0xFFFFFFFFU, part, o); }
    if ((threadIdx.x & 31U) == 0U) { atomicAdd(loss, part * scale); }
}

__global__ void gelu_bwd_kernel(const float* dA, const float* Z, __nv_bfloat16* dZ, std::size_t total) {
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < total;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x) {
        // dA arrives in FP32 from the GEMM and is rounded to BF16 like every activation gradient
        const float da = __bfloat162float(__float2bfloat16_rn(dA[i]));
        dZ[i] = __float2bfloat16_rn(da * gelu_grad(Z[i]));
    }
}

__global__ void bias_grad_kernel(const __nv_bfloat16* dZ, float* db, int M, int N) {
    const int n = static_cast<int>(blockIdx.x * blockDim.x + threadIdx.x);
    if (n >= N) { return; }
    float s = 0.f;
    for (int m = 0; m < M; ++m) { s += __bfloat162float(dZ[static_cast<std::size_t>(m) * N + n]); }
    db[n] = s;
}

__global__ void to_bf16_kernel(const float* x, __nv_bfloat16* y, std::size_t n) {
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x) {
        y[i] = __float2bfloat16_rn(x[i]);
    }
}

// Rows idx[0..B) of x [.][in] (BF16) and y [.][out] (FP32) into a batch.
__global__ void gather_kernel(const float* x, const float* y, const int* idx, int B, int in, int out, __nv_bfloat16* xb,
                              float* yb) {
    const std::size_t total_x = static_cast<std::size_t>(B) * in;
    const std::size_t total_y = static_cast<std::size_t>(B) * out;
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < total_x + total_y;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x) {
        if (i < total_x) {
            const std::size_t r = i / in;
            xb[i] = __float2bfloat16_rn(x[static_cast<std::size_t>(idx[r]) * in + i % in]);
        } else {
            const std::size_t j = i - total_x;
            const std::size_t r = j / out;
            yb[j] = y[static_cast<std::size_t>(idx[r]) * out + j % out];
        }
    }
}

__global__ void adam_kernel(float* w, const float* g, float* m, float* v, __nv_bfloat16* w16, std::size_t n, float lr,
                            float c1, float c2) {
    for (std::size_t i = blockIdx.x * static_cast<std::size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<std::size_t>(gridDim.x) * blockDim.x) {
        const float gi = g[i];
        const float mi = 0.9f * m[i] + 0.1f * gi;
        const float vi = 0.999f * v[i] + 0.001f * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
        w[i] = wi;
        w16[i] = __float2bfloat16_rn(wi);
    }
}

int grid_for(std::size_t n) { return static_cast<int>(std::min<std::size_t>((n + 255) / 256, 4096)); }

}// namespace

struct Mlp::Impl {
    int L{ 0 };
    std::vector<std::size_t> w_off, b_off;// offsets of W_l and b_l in the parameter arrays
    DevArray<float> master, grad, m1, m2;
    DevArray<__nv_bfloat16> w16;
    // per batch row capacity
    int cap{ 0 };
    std::vector<DevArray<__nv_bfloat16>> act;// act[l]: input of layer l, [B][widths[l]]
    std::vector<DevArray<float>> z;          // z[l]: pre-activation of layer l, [B][widths[l+1]]
    DevArray<float> c, dact;                 // GEMM output, activation gradient (FP32)
    DevArray<__nv_bfloat16> dz;              // pre-activation gradient (BF16)
    DevArray<float> target, loss;
    DevArray<int> idx;
    DevArray<float> xall, yall;
    std::uint64_t t{ 0 };                    // Adam steps
    cudaStream_t s{ nullptr };
};

Mlp::Mlp(const std::vector<int>& widths, std::uint64_t seed) : widths_{ widths }, impl_{ std::make_unique<Impl>() } {
    if (widths.size() < 2) { throw std::invalid_argument("an MLP needs at least an input and an output width"); }
    for (int w : widths) {
        if (w < 1 || w > 65536) { throw std::invalid_argument("layer widths must be in 1..65536"); }
    }
    Impl& I = *impl_;
    I.L = static_cast<int>(widths.size()) - 1;
    std::size_t off = 0;
    for (int l = 0; l < I.L; ++l) {
        I.w_off.push_back(off);
        off += static_cast<std::size_t>(widths[l]) * widths[l + 1];
        I.b_off.push_back(off);
        off += static_cast<std::size_t>(widths[l + 1]);
    }
    n_params_ = off;
    std::vector<float> p(off, 0.f);
    std::mt19937_64 rng(seed ^ 0x6D6C70ULL);
    for (int l = 0; l < I.L; ++l) {
        std::normal_distribution<float> nd(0.f, 1.f / std::sqrt(static_cast<float>(widths[l])));
        for (std::size_t i = 0; i < static_cast<std::size_t>(widths[l]) * widths[l + 1]; ++i) { p[I.w_off[l] + i] = nd(rng); }
    }
    I.master.resize(off);
    I.grad.resize(off);
    I.m1.resize(off);
    I.m2.resize(off);
    I.w16.resize(off);
    check(cudaStreamCreateWithFlags(&I.s, cudaStreamNonBlocking), "stream");
    set_params(p.data());
    check(cudaMemsetAsync(I.m1.p, 0, off * sizeof(float), I.s), "memset");
    check(cudaMemsetAsync(I.m2.p, 0, off * sizeof(float), I.s), "memset");
    check(cudaStreamSynchronize(I.s), "mlp init");
}

Mlp::~Mlp() {
    if (impl_ && impl_->s != nullptr) { cudaStreamDestroy(impl_->s); }
}

void Mlp::get_params(float* out) const {
    check(cudaMemcpy(out, impl_->master.p, n_params_ * sizeof(float), cudaMemcpyDeviceToHost), "copy params");
}

void Mlp::set_params(const float* in) {
    Impl& I = *impl_;
    check(cudaMemcpyAsync(I.master.p, in, n_params_ * sizeof(float), cudaMemcpyHostToDevice, I.s), "upload params");
    to_bf16_kernel<<<grid_for(n_params_), 256, 0, I.s>>>(I.master.p, I.w16.p, n_params_);
    check(cudaGetLastError(), "to_bf16");
    check(cudaStreamSynchronize(I.s), "set params");
}

namespace {

void gemm(const __nv_bfloat16* A, const __nv_bfloat16* B, float* C, int M, int N, int K, bool tA, bool tB, cudaStream_t s) {
    const dim3 grid(static_cast<unsigned>((N + kBN - 1) / kBN), static_cast<unsigned>((M + kBM - 1) / kBM));
    gemm_kernel<<<grid, 128, 0, s>>>(A, B, C, M, N, K, tA, tB);
}

// Buffers for batches of up to B rows.
void reserve(Mlp::Impl& I, const std::vector<int>& widths, int B) {
    if (B <= I.cap) { return; }
    const int maxw = *std::max_element(widths.begin(), widths.end());
    I.act.clear();
    I.z.clear();
    I.act.resize(static_cast<std::size_t>(I.L));
    I.z.resize(static_cast<std::size_t>(I.L));
    for (int l = 0; l < I.L; ++l) {
        I.act[static_cast<std::size_t>(l)].resize(static_cast<std::size_t>(B) * widths[l]);
        I.z[static_cast<std::size_t>(l)].resize(static_cast<std::size_t>(B) * widths[l + 1]);
    }
    I.c.resize(static_cast<std::size_t>(B) * maxw);
    I.dact.resize(static_cast<std::size_t>(B) * maxw);
    I.dz.resize(static_cast<std::size_t>(B) * maxw);
    I.target.resize(static_cast<std::size_t>(B) * widths.back());
    I.loss.resize(1);
    I.idx.resize(static_cast<std::size_t>(B));
    I.cap = B;
}

// Forward pass over B rows already in act[0]; the output lands in z[L-1].
void forward(Mlp::Impl& I, const std::vector<int>& widths, int B) {
    for (int l = 0; l < I.L; ++l) {
        const int in = widths[l];
        const int out = widths[l + 1];
        gemm(I.act[static_cast<std::size_t>(l)].p, I.w16.p + I.w_off[l], I.c.p, B, out, in, false, false, I.s);
        const bool hidden = l + 1 < I.L;
        __nv_bfloat16* next = hidden ? I.act[static_cast<std::size_t>(l + 1)].p : nullptr;
        bias_act_kernel<<<grid_for(static_cast<std::size_t>(B) * out), 256, 0, I.s>>>(
            I.c.p, I.master.p + I.b_off[l], I.z[static_cast<std::size_t>(l)].p, next, B, out, hidden);
    }
}

// Loss of the batch against I.target and the gradient of every parameter into I.grad.
void backward(Mlp::Impl& I, const std::vector<int>& widths, int B) {
    const int outw = widths.back();
    const std::size_t total = static_cast<std::size_t>(B) * outw;
    check(cudaMemsetAsync(I.loss.p, 0, sizeof(float), I.s), "memset loss");
    mse_kernel<<<grid_for(total), 256, 0, I.s>>>(I.z[static_cast<std::size_t>(I.L - 1)].p, I.target.p, I.dz.p, total,
                                                  1.f / static_cast<float>(total), I.loss.p);
    for (int l = I.L - 1; l >= 0; --l) {
        const int in = widths[l];
        const int out = widths[l + 1];
        // dW = act^T dZ, db = column sums of dZ
        gemm(I.act[static_cast<std::size_t>(l)].p, I.dz.p, I.grad.p + I.w_off[l], in, out, B, true, false, I.s);
        bias_grad_kernel<<<(out + 255) / 256, 256, 0, I.s>>>(I.dz.p, I.grad.p + I.b_off[l], B, out);
        if (l == 0) { break; }
        // dA = dZ W^T, then dZ of the layer below through GELU
        gemm(I.dz.p, I.w16.p + I.w_off[l], I.dact.p, B, in, out, false, true, I.s);
        gelu_bwd_kernel<<<grid_for(static_cast<std::size_t>(B) * in), 256, 0, I.s>>>(
            I.dact.p, I.z[static_cast<std::size_t>(l - 1)].p, I.dz.p, static_cast<std::size_t>(B) * in);
    }
}

}// namespace

float Mlp::gradients(const float* x, const float* y, int n, float* grads) {
    Impl& I = *impl_;
    if (n < 1) { throw std::invalid_argument("no rows"); }
    reserve(I, widths_, n);
    DevArray<float> xf(static_cast<std::size_t>(n) * widths_.front());
    check(cudaMemcpyAsync(xf.p, x, xf.n * sizeof(float), cudaMemcpyHostToDevice, I.s), "upload x");
    to_bf16_kernel<<<grid_for(xf.n), 256, 0, I.s>>>(xf.p, I.act[0].p, xf.n);
    check(cudaMemcpyAsync(I.target.p, y, static_cast<std::size_t>(n) * widths_.back() * sizeof(float), cudaMemcpyHostToDevice, I.s),
          "upload y");
    forward(I, widths_, n);
    backward(I, widths_, n);
    check(cudaGetLastError(), "mlp kernels");
    float loss = 0.f;
    check(cudaMemcpyAsync(&loss, I.loss.p, sizeof(float), cudaMemcpyDeviceToHost, I.s), "copy loss");
    if (grads != nullptr) {
        check(cudaMemcpyAsync(grads, I.grad.p, n_params_ * sizeof(float), cudaMemcpyDeviceToHost, I.s), "copy grads");
    }
    check(cudaStreamSynchronize(I.s), "mlp gradients");
    return loss;
}

float Mlp::train(const float* x, const float* y, int n, int batch, int epochs, float lr, std::uint64_t seed) {
    Impl& I = *impl_;
    if (n < 1 || batch < 1 || epochs < 0) { throw std::invalid_argument("bad training arguments"); }
    const int in = widths_.front();
    const int out = widths_.back();
    const int B = std::min(batch, n);
    reserve(I, widths_, B);
    I.xall.resize(static_cast<std::size_t>(n) * in);
    I.yall.resize(static_cast<std::size_t>(n) * out);
    check(cudaMemcpyAsync(I.xall.p, x, static_cast<std::size_t>(n) * in * sizeof(float), cudaMemcpyHostToDevice, I.s), "upload x");
    check(cudaMemcpyAsync(I.yall.p, y, static_cast<std::size_t>(n) * out * sizeof(float), cudaMemcpyHostToDevice, I.s), "upload y");
    std::vector<int> order(static_cast<std::size_t>(n));
    std::iota(order.begin(), order.end(), 0);
    std::mt19937_64 rng(seed);
    float epoch_loss = 0.f;
    std::vector<float> losses;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(order.begin(), order.end(), rng);
        double sum = 0.;
        int batches = 0;
        for (int b0 = 0; b0 + B <= n; b0 += B) {// whole batches only
            check(cudaMemcpyAsync(I.idx.p, order.data() + b0, static_cast<std::size_t>(B) * sizeof(int), cudaMemcpyHostToDevice, I.s),
                  "upload batch");
            gather_kernel<<<grid_for(static_cast<std::size_t>(B) * (in + out)), 256, 0, I.s>>>(I.xall.p, I.yall.p, I.idx.p, B, in,
                                                                                            out, I.act[0].p, I.target.p);
            forward(I, widths_, B);
            backward(I, widths_, B);
            ++I.t;
            const float c1 = 1.f - std::pow(0.9f, static_cast<float>(I.t));
            const float c2 = 1.f - std::pow(0.999f, static_cast<float>(I.t));
            adam_kernel<<<grid_for(n_params_), 256, 0, I.s>>>(I.master.p, I.grad.p, I.m1.p, I.m2.p, I.w16.p, n_params_, lr, c1, c2);
            float l = 0.f;
            check(cudaMemcpyAsync(&l, I.loss.p, sizeof(float), cudaMemcpyDeviceToHost, I.s), "copy loss");
            check(cudaStreamSynchronize(I.s), "mlp step");
            sum += l;
            ++batches;
        }
        check(cudaGetLastError(), "mlp kernels");
        epoch_loss = batches > 0 ? static_cast<float>(sum / batches) : 0.f;
    }
    return epoch_loss;
}

void Mlp::predict(const float* x, int n, float* y) {
    Impl& I = *impl_;
    if (n < 1) { return; }
    const int in = widths_.front();
    const int out = widths_.back();
    const int B = std::min(n, 1024);
    reserve(I, widths_, B);
    DevArray<float> xf(static_cast<std::size_t>(B) * in);
    for (int r0 = 0; r0 < n; r0 += B) {
        const int b = std::min(B, n - r0);
        check(cudaMemcpyAsync(xf.p, x + static_cast<std::size_t>(r0) * in, static_cast<std::size_t>(b) * in * sizeof(float),
                              cudaMemcpyHostToDevice, I.s),
              "upload x");
        to_bf16_kernel<<<grid_for(static_cast<std::size_t>(b) * in), 256, 0, I.s>>>(xf.p, I.act[0].p, static_cast<std::size_t>(b) * in);
        forward(I, widths_, b);
        check(cudaMemcpyAsync(y + static_cast<std::size_t>(r0) * out, I.z[static_cast<std::size_t>(I.L - 1)].p,
                              static_cast<std::size_t>(b) * out * sizeof(float), cudaMemcpyDeviceToHost, I.s),
              "copy y");
    }
    check(cudaGetLastError(), "mlp kernels");
    check(cudaStreamSynchronize(I.s), "mlp predict");
}

}// namespace psim::gpu
