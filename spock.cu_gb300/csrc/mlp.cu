// Learned warm start: a small MLP trained and evaluated on the GPU by these kernels.
//
// The network maps an initial state x0 (nIn values) to the coefficients of a solution basis:
//   A1 = W1 X + b1, H1 = gelu(A1);  A2 = W2 H1 + b2, H2 = gelu(A2);  Y = W3 H2 + b3,
// columns = samples.  Weights live as FP32 master copies (for Adam) and BF16 copies that every
// product reads; all products (forward, and both gradient products of the backward pass) run on
// the tcgen05 tensor cores (umma_gemm.cu) with FP32 accumulation, activations and gradients
// entering as hi + lo BF16 pairs.  GELU is the tanh form
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
#include "umma_gemm.hpp"

namespace spock {

namespace {

#define MCK(x)                                                                                     \
    do {                                                                                           \
        cudaError_t e_ = (x);                                                                      \
        if (e_ != cudaSuccess)                                                                     \
            throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + \
                                     __FILE__ + ":" + std::to_string(__LINE__));                   \
    } while (0)


__device__ __forceinline__ float geluTanh(float a, float *dgelu) {
    const float c = 0.7978845608028654f, u = c * (a + 0.044715f * a * a * a);
    const float t = tanhf(u);
    if (dgelu) *dgelu = 0.5f * (1.f + t) + 0.5f * a * (1.f - t * t) * c * (1.f + 3.f * 0.044715f * a * a);
    return 0.5f * a * (1.f + t);
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
__global__ void k_adam(float *w, const float *g, float *mo, float *v, size_t n, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const float gg = g[e];
        const float m1 = b1 * mo[e] + (1.f - b1) * gg, v1 = b2 * v[e] + (1.f - b2) * gg * gg;
        mo[e] = m1;
        v[e] = v1;
        const float nw = w[e] - lr * (m1 / c1) / (sqrtf(v1 / c2) + eps);
        w[e] = nw;
    }
}

int grid1(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 8); }

// BF16 operand copies for the tensor-core GEMMs (umma_gemm.cu: D = A B', both K-major).  An
// FP32 matrix is split into hi = bf16(x) and lo = bf16(x - hi), which together carry about 16
// bits of mantissa; the K dimension of an operand is then a concatenation of segments of 64-
// padded length, each hi or lo, so one GEMM sums hi*hi + lo*hi (+ hi*lo) products: the weights
// (BF16 by design) meet activations and gradients at close to FP32 accuracy.
// Segment j of an operand row is lo when bit j of `loMask` is set, hi otherwise.

// Rows: src (rows x d, row-major, FP32) -> dst (rows x nseg*dP, BF16), zero past column d.
__global__ void k_split_rows(const float *src, int rows, int d, __nv_bfloat16 *dst, int dP, int nseg, int loMask) {
    const size_t n = (size_t)rows * dP;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / dP), c = (int)(e % dP);
        const float x = c < d ? src[(size_t)r * d + c] : 0.f;
        const __nv_bfloat16 hi = __float2bfloat16_rn(x), lo = __float2bfloat16_rn(x - __bfloat162float(hi));
        for (int j = 0; j < nseg; j++) dst[(size_t)r * nseg * dP + (size_t)j * dP + c] = (loMask >> j) & 1 ? lo : hi;
    }
}

// Transposed: src (rows x d, row-major, FP32) -> dst (d x nseg*rP, BF16), dst[c][j*rP + r] the
// hi or lo part of src[r][c], zero for r >= rows.  32 x 32 tiles through shared memory.
__global__ void k_split_cols(const float *src, int rows, int d, __nv_bfloat16 *dst, int rP, int nseg, int loMask) {
    __shared__ float t[32][33];
    const int r0 = blockIdx.x * 32, c0 = blockIdx.y * 32, tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    for (int k = ty; k < 32; k += 8) {
        const int r = r0 + k, c = c0 + tx;
        t[k][tx] = (r < rows && c < d) ? src[(size_t)r * d + c] : 0.f;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int c = c0 + k, r = r0 + tx;
        if (c >= d || r >= rP) continue;
        const float x = t[tx][k];
        const __nv_bfloat16 hi = __float2bfloat16_rn(x), lo = __float2bfloat16_rn(x - __bfloat162float(hi));
        for (int j = 0; j < nseg; j++) dst[(size_t)c * nseg * rP + (size_t)j * rP + r] = (loMask >> j) & 1 ? lo : hi;
    }
}

// The weights' BF16 operands from the FP32 master W (out x in, column-major):
//   row form  (forward, B of X W'):      wr[o][j*inP + i] = bf16(W[o][i]), two equal segments;
//   column form (backward, B of dA W):   wc[i][j*outP + o] = bf16(W[o][i]), two equal segments.
__global__ void k_weight_ops(const float *W, int out, int in, __nv_bfloat16 *wr, int inP, __nv_bfloat16 *wc, int outP) {
    const size_t n = (size_t)out * in;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int o = (int)(e % out), i = (int)(e / out);
        const __nv_bfloat16 v = __float2bfloat16_rn(W[e]);
        for (int j = 0; j < 2; j++) {
            wr[(size_t)o * 2 * inP + (size_t)j * inP + i] = v;
            if (wc) wc[(size_t)i * 2 * outP + (size_t)j * outP + o] = v;
        }
    }
}

inline int pad64(int v) { return (v + 63) & ~63; }

}  // namespace


// Three layers: sizes d0 -> d1 -> d2 -> d3.  Parameters packed as W1 (d1 x d0), b1, W2 (d2 x d1),
// b2, W3 (d3 x d2), b3 in one FP32 array (column-major W's: the Adam master copy).  Every product
// runs on the tensor cores (gemmBf16): samples are rows (an activation "d x cols, column-major"
// is "cols x d, row-major"), weights enter as BF16, activations and gradients as hi + lo BF16
// pairs, accumulation in FP32.
struct Mlp {
    int d[4], dP[4];
    size_t off[6], total;
    float *w = nullptr, *g = nullptr, *mo = nullptr, *v = nullptr;
    __nv_bfloat16 *wr[3] = {}, *wc[3] = {};  // weight operands (row and column forms)
    int cap = 0;                              // columns the activations are allocated for
    float *A1 = nullptr, *H1 = nullptr, *A2 = nullptr, *H2 = nullptr, *Y = nullptr, *dY = nullptr, *dH = nullptr,
          *loss = nullptr;
    __nv_bfloat16 *opA = nullptr, *opB = nullptr;  // activation / gradient operands
    int *err = nullptr;
    long steps = 0;
    cudaStream_t st = nullptr;

    Mlp(int d0, int d1, int d2, int d3) {
        d[0] = d0; d[1] = d1; d[2] = d2; d[3] = d3;
        for (int q = 0; q < 4; q++) dP[q] = pad64(d[q]);
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
        for (int l = 0; l < 3; l++) {
            MCK(cudaMalloc(&wr[l], sizeof(__nv_bfloat16) * (size_t)d[l + 1] * 2 * dP[l]));
            MCK(cudaMemset(wr[l], 0, sizeof(__nv_bfloat16) * (size_t)d[l + 1] * 2 * dP[l]));
            if (l > 0) {
                MCK(cudaMalloc(&wc[l], sizeof(__nv_bfloat16) * (size_t)d[l] * 2 * dP[l + 1]));
                MCK(cudaMemset(wc[l], 0, sizeof(__nv_bfloat16) * (size_t)d[l] * 2 * dP[l + 1]));
            }
        }
        MCK(cudaMalloc(&loss, sizeof(float)));
        MCK(cudaMalloc(&err, sizeof(int)));
        MCK(cudaMemset(err, 0, sizeof(int)));
    }
    ~Mlp() {
        for (void *p : {(void *)w, (void *)g, (void *)mo, (void *)v, (void *)A1, (void *)H1, (void *)A2, (void *)H2,
                        (void *)Y, (void *)dY, (void *)dH, (void *)loss, (void *)opA, (void *)opB, (void *)err})
            cudaFree(p);
        for (int l = 0; l < 3; l++) {
            cudaFree(wr[l]);
            cudaFree(wc[l]);
        }
        if (st) cudaStreamDestroy(st);
    }
    void reserve(int cols) {
        if (cols <= cap) return;
        for (void *p : {(void *)A1, (void *)H1, (void *)A2, (void *)H2, (void *)Y, (void *)dY, (void *)dH, (void *)opA,
                        (void *)opB})
            cudaFree(p);
        const int wmax = std::max(d[1], d[2]);
        MCK(cudaMalloc(&A1, sizeof(float) * (size_t)d[1] * cols));
        MCK(cudaMalloc(&H1, sizeof(float) * (size_t)d[1] * cols));
        MCK(cudaMalloc(&A2, sizeof(float) * (size_t)d[2] * cols));
        MCK(cudaMalloc(&H2, sizeof(float) * (size_t)d[2] * cols));
        MCK(cudaMalloc(&Y, sizeof(float) * (size_t)d[3] * cols));
        MCK(cudaMalloc(&dY, sizeof(float) * (size_t)d[3] * cols));
        MCK(cudaMalloc(&dH, sizeof(float) * (size_t)wmax * cols));
        // operands: rows x 2 dP (forward / backward data) or d x 3 colsP (weight gradients)
        size_t ops = 0;
        for (int q = 0; q < 4; q++) ops = std::max({ops, (size_t)cols * 2 * dP[q], (size_t)d[q] * 3 * pad64(cols)});
        MCK(cudaMalloc(&opA, sizeof(__nv_bfloat16) * ops));
        MCK(cudaMalloc(&opB, sizeof(__nv_bfloat16) * ops));
        cap = cols;
    }
    void refreshBf16() {
        for (int l = 0; l < 3; l++) {
            k_weight_ops<<<grid1((size_t)d[l + 1] * d[l]), 256, 0, st>>>(w + off[2 * l], d[l + 1], d[l], wr[l], dP[l], wc[l],
                                                                        dP[l + 1]);
            MCK(cudaGetLastError());
        }
    }
    const float *b(int l) const { return w + off[2 * l + 1]; }

    void gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, int K, GemmEpilogue E) {
        E.err = err;
        gemmBf16(A, B, M, N, K, E, st);
    }
    // [hi | lo] rows of an activation (rows x d) as the A operand of a product with weights
    void splitRows(const float *src, int rows, int dd, __nv_bfloat16 *dst) {
        k_split_rows<<<grid1((size_t)rows * pad64(dd)), 256, 0, st>>>(src, rows, dd, dst, pad64(dd), 2, 0b10);
        MCK(cudaGetLastError());
    }
    // transposed three-segment operands of a weight gradient: A = [hi|lo|hi], B = [hi|hi|lo]
    void splitCols(const float *src, int rows, int dd, __nv_bfloat16 *dst, int loMask) {
        dim3 grid((unsigned)((pad64(rows) + 31) / 32), (unsigned)((dd + 31) / 32));
        k_split_cols<<<grid, 256, 0, st>>>(src, rows, dd, dst, pad64(rows), 3, loMask);
        MCK(cudaGetLastError());
    }
    void checkErr() {
        int h = 0;
        MCK(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, st));
        MCK(cudaStreamSynchronize(st));
        if (h) throw std::runtime_error("[mlp] the tensor-core pipeline gave up (code " + std::to_string(h) + ")");
    }

    // layer l: out (cols x d[l+1]) = in (cols x d[l]) W' + b, and its GELU when act
    void layer(int l, const float *in, int cols, float *pre, float *act) {
        splitRows(in, cols, d[l], opA);
        GemmEpilogue E;
        E.colAdd = b(l);
        E.D = pre;
        E.ldd = d[l + 1];
        if (act) {
            E.gelu = 1;
            E.Dact = act;
        }
        gemm(opA, wr[l], cols, d[l + 1], 2 * dP[l], E);
    }

    void forward(const float *X, int cols) {
        reserve(cols);
        layer(0, X, cols, A1, H1);
        layer(1, H1, cols, A2, H2);
        layer(2, H2, cols, Y, nullptr);
    }

    // dW of layer l (column-major d[l+1] x d[l], i.e. row-major d[l] x d[l+1]) = sum over samples of
    // in[s][i] dA[s][o], into g.
    void weightGrad(int l, const float *in, const float *dA, int cols) {
        splitCols(in, cols, d[l], opA, 0b010);
        splitCols(dA, cols, d[l + 1], opB, 0b100);
        GemmEpilogue E;
        E.D = g + off[2 * l];
        E.ldd = d[l + 1];
        gemm(opA, opB, d[l], d[l + 1], 3 * pad64(cols), E);
        k_rowsum<<<(d[l + 1] + 255) / 256, 256, 0, st>>>(dA, g + off[2 * l + 1], d[l + 1], cols);
        MCK(cudaGetLastError());
    }
    // dH (cols x d[l]) = dA (cols x d[l+1]) W_l
    void dataGrad(int l, const float *dA, int cols, float *out) {
        splitRows(dA, cols, d[l + 1], opA);
        GemmEpilogue E;
        E.D = out;
        E.ldd = d[l];
        gemm(opA, wc[l], cols, d[l], 2 * dP[l + 1], E);
    }

    // Gradients of the mean squared error into g (same packing as w); returns the loss.
    float backward(const float *X, const float *T, int cols) {
        MCK(cudaMemsetAsync(loss, 0, sizeof(float), st));
        k_mse<<<grid1((size_t)d[3] * cols), 256, 0, st>>>(Y, T, dY, d[3], cols, loss);
        MCK(cudaGetLastError());
        weightGrad(2, H2, dY, cols);
        dataGrad(2, dY, cols, dH);
        k_gelu_back<<<grid1((size_t)d[2] * cols), 256, 0, st>>>(dH, A2, (size_t)d[2] * cols);  // dA2
        MCK(cudaGetLastError());
        weightGrad(1, H1, dH, cols);
        dataGrad(1, dH, cols, dH);  // the operand copy of dA2 is taken before dH is overwritten
        k_gelu_back<<<grid1((size_t)d[1] * cols), 256, 0, st>>>(dH, A1, (size_t)d[1] * cols);  // dA1
        MCK(cudaGetLastError());
        weightGrad(0, X, dH, cols);
        float l = 0.f;
        MCK(cudaMemcpyAsync(&l, loss, sizeof(float), cudaMemcpyDeviceToHost, st));
        checkErr();
        return l;
    }

    void adam(float lr) {
        steps++;
        const float b1 = .9f, b2 = .999f;
        const float c1 = 1.f - powf(b1, (float)steps), c2 = 1.f - powf(b2, (float)steps);
        k_adam<<<grid1(total), 256, 0, st>>>(w, g, mo, v, total, lr, b1, b2, 1e-8f, c1, c2);
        MCK(cudaGetLastError());
        refreshBf16();
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
        m.checkErr();
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
