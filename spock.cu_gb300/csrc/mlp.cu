// Learned warm start: a small MLP trained and evaluated on the GPU by these kernels.
//
// The network maps an initial state x0 (nIn values) to the coefficients of a solution basis:
//   A1 = W1 X + b1, H1 = gelu(A1);  A2 = W2 H1 + b2, H2 = gelu(A2);  Y = W3 H2 + b3,
// columns = samples.  Weights live as FP32 master copies (for Adam) and BF16 copies that the
// forward products read; every product accumulates in FP32.  GELU is the tanh form
// 0.5 a (1 + tanh(sqrt(2/pi) (a + 0.044715 a^3))).
//
// C-ABI (spock_gb300.h): spock_mlp_create / _free / _set_params / _get_params / _forward /
// _train_step; all tensors are column-major device arrays, samples in columns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/spock_gb300.h"
#include "capi_internal.hpp"

namespace spock {

namespace {

#define MCK(x)                                                                                     \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + \
                                     __FILE__ + ":" + std::to_string(__LINE__));                   \
    } while (0)

__device__ __forceinline__ float ld(const float *p, size_t i) { return p[i]; }
__device__ __forceinline__ float ld(const __nv_bfloat16 *p, size_t i) { return __bfloat162float(p[i]); }

// C[m x n] = alpha * op(A)[m x k] op(B)[k x n] + beta * C, column-major with leading dimensions;
// op transposes when tA / tB.  64 x 64 tiles, 256 threads with 4 x 4 outputs each, operands
// staged through shared memory in 16-wide slabs, FP32 accumulation.
constexpr int kBM = 64, kBN = 64, kBK = 16;

template <typename TA, typename TB>
__global__ void __launch_bounds__(256) k_gemm(int m, int n, int k, float alpha, const TA *A, int lda, bool tA,
                                              const TB *B, int ldb, bool tB, float beta, float *C, int ldc) {
    __shared__ float sA[kBK][kBM + 4];
    __shared__ float sB[kBK][kBN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < k; k0 += kBK) {
        for (int e = threadIdx.x; e < kBK * kBM; e += 256) {  // sA[kk][i] = op(A)(m0 + i, k0 + kk)
            const int kk = e / kBM, i = e % kBM, r = m0 + i, c = k0 + kk;
            float v = 0.f;
            if (r < m && c < k) v = tA ? ld(A, (size_t)r * lda + c) : ld(A, (size_t)c * lda + r);
            sA[kk][i] = v;
        }
        for (int e = threadIdx.x; e < kBK * kBN; e += 256) {  // sB[kk][j] = op(B)(k0 + kk, n0 + j)
            const int kk = e / kBN, j = e % kBN, r = k0 + kk, c = n0 + j;
            float v = 0.f;
            if (r < k && c < n) v = tB ? ld(B, (size_t)r * ldb + c) : ld(B, (size_t)c * ldb + r);
            sB[kk][j] = v;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kBK; kk++) {
            float a[4], bv[4];
#pragma unroll
            for (int q = 0; q < 4; q++) a[q] = sA[kk][ty * 4 + q];
#pragma unroll
            for (int q = 0; q < 4; q++) bv[q] = sB[kk][tx * 4 + q];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(a[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int r = m0 + ty * 4 + i, c = n0 + tx * 4 + j;
            if (r < m && c < n) {
                float *o = C + (size_t)c * ldc + r;
                *o = alpha * acc[i][j] + (beta != 0.f ? beta * *o : 0.f);
            }
        }
}

__device__ __forceinline__ float geluTanh(float a, float *dgelu) {
    const float c = 0.7978845608028654f, u = c * (a + 0.044715f * a * a * a);
    const float t = tanhf(u);
    if (dgelu) *dgelu = 0.5f * (1.f + t) + 0.5f * a * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * a * a);
    return 0.5f * a * (1.f + t);
}

// A += b (per row); H = gelu(A) when act, else H = A.
__global__ void k_bias_act(float *A, float *H, const float *bias, int rows, int cols, int act) {
    const size_t n = (size_t)rows * cols;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float a = A[e] + bias[e % rows];
        A[e] = a;
        H[e] = act ? geluTanh(a, nullptr) : a;
    }
}

// dA = dH * gelu'(A), in place on dH.
__global__ void k_gelu_back(float *dH, const float *A, size_t n) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        float d;
        geluTanh(A[e], &d);
        dH[e] *= d;
    }
}

// dY = 2 (Y - T) / (rows * cols), and the loss sum of squares / (rows * cols) into *loss.
__global__ void k_mse(const float *Y, const float *T, float *dY, int rows, int cols, float *loss) {
    const size_t n = (size_t)rows * cols;
    float s = 0.f;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float d = Y[e] - T[e];
        dY[e] = 2.f * d / (float)n;
        s += d * d;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (float)n);
}

// db = sum over columns of dA.
__global__ void k_rowsum(const float *dA, float *db, int rows, int cols) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    float s = 0.f;
    for (int c = 0; c < cols; c++) s += dA[(size_t)c * rows + r];
    db[r] = s;
}

// Adam on FP32 master weights; refreshes the BF16 copy.
__global__ void k_adam(float *w, __nv_bfloat16 *wb, const float *g, float *mo, float *v, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float m1 = b1 * mo[e] + (1.f - b1) * gg, v1 = b2 * v[e] + (1.f - b2) * gg * gg;
        mo[e] = m1;
        v[e] = v1;
        const float nw = w[e] - lr * (m1 / c1) / (sqrtf(v1 / c2) + eps);
        w[e] = nw;
        if (wb) wb[e] = __float2bfloat16(nw);
    }
}

__global__ void k_to_bf16(const float *w, __nv_bfloat16 *wb, size_t n) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
        wb[e] = __float2bfloat16(w[e]);
}

int grid1(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 8); }

template <typename TA, typename TB>
void gemm(cudaStream_t st, int m, int n, int k, float alpha, const TA *A, int lda, bool tA, const TB *B, int ldb,
          bool tB, float beta, float *C, int ldc) {
    dim3 g((unsigned)((m + kBM - 1) / kBM), (unsigned)((n + kBN - 1) / kBN));
    k_gemm<TA, TB><<<g, 256, 0, st>>>(m, n, k, alpha, A, lda, tA, B, ldb, tB, beta, C, ldc);
    MCK(cudaGetLastError());
}

}  // namespace

// Three layers: sizes d0 -> d1 -> d2 -> d3.  Parameters packed as W1 (d1 x d0), b1, W2 (d2 x d1),
// b2, W3 (d3 x d2), b3 in one FP32 array (and a BF16 copy of the W's at the same offsets).
struct Mlp {
    int d[4];
    size_t off[6], total;
    float *w = nullptr, *g = nullptr, *mo = nullptr, *v = nullptr;
    __nv_bfloat16 *wb = nullptr;
    int cap = 0;  // columns the activations are allocated for
    float *A1 = nullptr, *H1 = nullptr, *A2 = nullptr, *H2 = nullptr, *Y = nullptr, *dY = nullptr, *dH = nullptr,
          *loss = nullptr;
    long steps = 0;
    cudaStream_t st = nullptr;

    Mlp(int d0, int d1, int d2, int d3) {
        d[0] = d0; d[1] = d1; d[2] = d2; d[3] = d3;
        size_t o = 0;
        for (int l = 0; l < 3; l++) {
            off[2 * l] = o;
            o += (size_t)d[l + 1] * d[l];
            off[2 * l + 1] = o;
            o += (size_t)d[l + 1];
        }
        total = o;
        MCK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        for (float **p : {&w, &g, &mo, &v}) {
            MCK(cudaMalloc(p, sizeof(float) * total));
            MCK(cudaMemset(*p, 0, sizeof(float) * total));
        }
        MCK(cudaMalloc(&wb, sizeof(__nv_bfloat16) * total));
        MCK(cudaMalloc(&loss, sizeof(float)));
    }
    ~Mlp() {
        for (void *p : {(void *)w, (void *)g, (void *)mo, (void *)v, (void *)wb, (void *)A1, (void *)H1, (void *)A2,
                        (void *)H2, (void *)Y, (void *)dY, (void *)dH, (void *)loss})
            cudaFree(p);
        if (st) cudaStreamDestroy(st);
    }
    void reserve(int cols) {
        if (cols <= cap) return;
        for (void *p : {(void *)A1, (void *)H1, (void *)A2, (void *)H2, (void *)Y, (void *)dY, (void *)dH}) cudaFree(p);
        const int wmax = std::max(d[1], d[2]);
        MCK(cudaMalloc(&A1, sizeof(float) * (size_t)d[1] * cols));
        MCK(cudaMalloc(&H1, sizeof(float) * (size_t)d[1] * cols));
        MCK(cudaMalloc(&A2, sizeof(float) * (size_t)d[2] * cols));
        MCK(cudaMalloc(&H2, sizeof(float) * (size_t)d[2] * cols));
        MCK(cudaMalloc(&Y, sizeof(float) * (size_t)d[3] * cols));
        MCK(cudaMalloc(&dY, sizeof(float) * (size_t)d[3] * cols));
        MCK(cudaMalloc(&dH, sizeof(float) * (size_t)wmax * cols));
        cap = cols;
    }
    void refreshBf16() {
        k_to_bf16<<<grid1(total), 256, 0, st>>>(w, wb, total);
        MCK(cudaGetLastError());
    }
    const __nv_bfloat16 *W(int l) const { return wb + off[2 * l]; }
    const float *b(int l) const { return w + off[2 * l + 1]; }

    void forward(const float *X, int cols) {
        reserve(cols);
        gemm(st, d[1], cols, d[0], 1.f, W(0), d[1], false, X, d[0], false, 0.f, A1, d[1]);
        k_bias_act<<<grid1((size_t)d[1] * cols), 256, 0, st>>>(A1, H1, b(0), d[1], cols, 1);
        gemm(st, d[2], cols, d[1], 1.f, W(1), d[2], false, H1, d[1], false, 0.f, A2, d[2]);
        k_bias_act<<<grid1((size_t)d[2] * cols), 256, 0, st>>>(A2, H2, b(1), d[2], cols, 1);
        gemm(st, d[3], cols, d[2], 1.f, W(2), d[3], false, H2, d[2], false, 0.f, Y, d[3]);
        k_bias_act<<<grid1((size_t)d[3] * cols), 256, 0, st>>>(Y, Y, b(2), d[3], cols, 0);
        MCK(cudaGetLastError());
    }

    // Gradients of the mean squared error into g (same packing as w); returns the loss.
    float backward(const float *X, const float *T, int cols) {
        MCK(cudaMemsetAsync(loss, 0, sizeof(float), st));
        k_mse<<<grid1((size_t)d[3] * cols), 256, 0, st>>>(Y, T, dY, d[3], cols, loss);
        // layer 3: dW3 = dY H2', db3 = rowsum dY, dH2 = W3' dY
        gemm(st, d[3], d[2], cols, 1.f, dY, d[3], false, H2, d[2], true, 0.f, g + off[4], d[3]);
        k_rowsum<<<(d[3] + 255) / 256, 256, 0, st>>>(dY, g + off[5], d[3], cols);
        gemm(st, d[2], cols, d[3], 1.f, W(2), d[3], true, dY, d[3], false, 0.f, dH, d[2]);
        k_gelu_back<<<grid1((size_t)d[2] * cols), 256, 0, st>>>(dH, A2, (size_t)d[2] * cols);
        // layer 2: dW2 = dA2 H1', db2, dH1 = W2' dA2 (dA2 is kept in A2's place after use)
        gemm(st, d[2], d[1], cols, 1.f, dH, d[2], false, H1, d[1], true, 0.f, g + off[2], d[2]);
        k_rowsum<<<(d[2] + 255) / 256, 256, 0, st>>>(dH, g + off[3], d[2], cols);
        MCK(cudaMemcpyAsync(A2, dH, sizeof(float) * (size_t)d[2] * cols, cudaMemcpyDeviceToDevice, st));
        gemm(st, d[1], cols, d[2], 1.f, W(1), d[2], true, A2, d[2], false, 0.f, dH, d[1]);
        k_gelu_back<<<grid1((size_t)d[1] * cols), 256, 0, st>>>(dH, A1, (size_t)d[1] * cols);
        // layer 1: dW1 = dA1 X', db1
        gemm(st, d[1], d[0], cols, 1.f, dH, d[1], false, X, d[0], true, 0.f, g + off[0], d[1]);
        k_rowsum<<<(d[1] + 255) / 256, 256, 0, st>>>(dH, g + off[1], d[1], cols);
        MCK(cudaGetLastError());
        float l = 0.f;
        MCK(cudaMemcpyAsync(&l, loss, sizeof(float), cudaMemcpyDeviceToHost, st));
        MCK(cudaStreamSynchronize(st));
        return l;
    }

    void adam(float lr) {
        steps++;
        const float b1 = .9f, b2 = .999f;
        const float c1 = 1.f - powf(b1, (float)steps), c2 = 1.f - powf(b2, (float)steps);
        k_adam<<<grid1(total), 256, 0, st>>>(w, wb, g, mo, v, total, lr, b1, b2, 1e-8f, c1, c2);
        MCK(cudaGetLastError());
    }
};

}  // namespace spock

struct spock_mlp_s {
    std::unique_ptr<spock::Mlp> m;
};

extern "C" {

int spock_mlp_create(const int *dims4, int device, spock_mlp *out) {
    return spock::guardedCall([&] {
        if (!dims4 || !out) throw std::invalid_argument("[mlp] null argument");
        for (int q = 0; q < 4; q++)
            if (dims4[q] < 1) throw std::invalid_argument("[mlp] layer sizes must be positive");
        MCK(cudaSetDevice(device));
        auto *h = new spock_mlp_s;
        h->m = std::make_unique<spock::Mlp>(dims4[0], dims4[1], dims4[2], dims4[3]);
        *out = h;
    });
}

void spock_mlp_free(spock_mlp h) { delete h; }

long spock_mlp_param_count(spock_mlp h) { return h ? (long)h->m->total : 0; }

int spock_mlp_set_params(spock_mlp h, const float *params) {
    return spock::guardedCall([&] {
        if (!h || !params) throw std::invalid_argument("[mlp] null argument");
        MCK(cudaMemcpy(h->m->w, params, sizeof(float) * h->m->total, cudaMemcpyHostToDevice));
        h->m->refreshBf16();
        MCK(cudaStreamSynchronize(h->m->st));
    });
}

int spock_mlp_get_params(spock_mlp h, float *params, float *grads) {
    return spock::guardedCall([&] {
        if (!h) throw std::invalid_argument("[mlp] null argument");
        MCK(cudaStreamSynchronize(h->m->st));
        if (params) MCK(cudaMemcpy(params, h->m->w, sizeof(float) * h->m->total, cudaMemcpyDeviceToHost));
        if (grads) MCK(cudaMemcpy(grads, h->m->g, sizeof(float) * h->m->total, cudaMemcpyDeviceToHost));
    });
}

int spock_mlp_forward(spock_mlp h, const void *x_device, int cols, void *y_device) {
    return spock::guardedCall([&] {
        if (!h || !x_device || !y_device || cols < 1) throw std::invalid_argument("[mlp] bad argument");
        spock::Mlp &m = *h->m;
        m.forward((const float *)x_device, cols);
        MCK(cudaMemcpyAsync(y_device, m.Y, sizeof(float) * (size_t)m.d[3] * cols, cudaMemcpyDeviceToDevice, m.st));
        MCK(cudaStreamSynchronize(m.st));
    });
}

int spock_mlp_train_step(spock_mlp h, const void *x_device, const void *t_device, int cols, float lr, float *loss) {
    return spock::guardedCall([&] {
        if (!h || !x_device || !t_device || cols < 1) throw std::invalid_argument("[mlp] bad argument");
        spock::Mlp &m = *h->m;
        m.forward((const float *)x_device, cols);
        const float l = m.backward((const float *)x_device, (const float *)t_device, cols);
        if (lr > 0.f) m.adam(lr);
        MCK(cudaStreamSynchronize(m.st));
        if (loss) *loss = l;
    });
}

}  // extern "C"
