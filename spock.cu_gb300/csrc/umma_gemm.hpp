// tcgen05 BF16 GEMM (umma_gemm.cu): D = alpha * A B' (+ rowAdd[m]) (+ colAdd[n]), optionally GELU.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace spock {

struct GemmEpilogue {
    float alpha = 1.f;
    const float *rowAdd = nullptr;  // [M], added to every row m (or null)
    const float *colAdd = nullptr;  // [N], added to every column n (or null)
    int gelu = 0;                   // GELU (tanh form) after the additions, for Dact and Dbf
    float *D = nullptr;             // FP32 row-major M x N before the GELU, leading dimension ldd (or null)
    double *D64 = nullptr;          // the same in FP64 (or null)
    float *Dact = nullptr;          // FP32 after the GELU, same layout (or null)
    long ldd = 0;
    __nv_bfloat16 *Dbf = nullptr;   // BF16 copy of the (activated) result, leading dimension lddBf (or null)
    long lddBf = 0;
    int *err = nullptr;             // device flag: nonzero when a pipeline wait gave up
};

// A: M x K, B: N x K, BF16 row-major (K contiguous), K a multiple of 64, 16-byte aligned.
// Launches on `stream`; throws std::invalid_argument on bad sizes.
void gemmBf16(const void *A, const void *B, long M, long N, int K, const GemmEpilogue &E, cudaStream_t stream);

}  // namespace spock
