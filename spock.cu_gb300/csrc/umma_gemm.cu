// BF16 GEMM on the 5th-generation tensor cores (tcgen05, sm_103a) for the learned warm start:
//   D[m][n] = alpha * sum_k A[m][k] B[n][k]  (+ rowAdd[m]) (+ colAdd[n])   (then optionally GELU)
// A (M x K) and B (N x K) are BF16, row-major with K contiguous ("K-major"), K a multiple of 64;
// accumulation is FP32 in tensor memory (TMEM).  Outputs: FP32 D (row-major, ldd), its GELU,
// and/or a BF16 copy, any of them optional.
//
// One CTA computes a 128 x 128 tile of D with four warps:
//  * warp 0, one lane: TMA producer.  Each K block of 64 brings a 128 x 64 slice of A and of B
//    into shared memory (cp.async.bulk.tensor, 128-byte swizzle) on a ring of kGStages stages
//    guarded by "full" / "empty" mbarriers;
//  * warp 1, one lane: issues tcgen05.mma (M = 128, N = 128, K = 16, both operands from shared
//    memory through matrix descriptors) into a 128-column TMEM accumulator, and tcgen05.commit
//    frees each stage and finally signals the epilogue;
//  * all four warps: epilogue, each warp reading its 32 TMEM lanes (= rows) with tcgen05.ld.
// Every mbarrier wait is bounded: after kSpinLimit polls the kernel records an error code in
// *err, stops issuing work, waits (bounded) for its own copies in flight, frees its TMEM and
// returns, so a fault in the pipeline ends the call with an error instead of a hung GPU.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <stdexcept>
#include <string>

#include "capi_internal.hpp"
#include "umma_gemm.hpp"

namespace spock {

namespace {

constexpr int kGM = 128, kGN = 128, kGK = 64, kGStages = 3, kGThreads = 128;
constexpr uint32_t kTileBytes = kGM * kGK * 2;  // one 128 x 64 BF16 slice: 16 KB
constexpr uint32_t kTmemCols = 128;
constexpr unsigned kSpinLimit = 1u << 24;
constexpr size_t kGemmSmem = 1024 + (size_t)kGStages * 2 * kTileBytes + 256;

// Instruction descriptor of tcgen05.mma kind::f16: D FP32 (bits 4-5 = 1), A and B BF16 (bits
// 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at 24-28.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kGN >> 3) << 17) | ((uint32_t)(kGM >> 4) << 24);

__device__ __forceinline__ uint32_t sAddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor of a K-major operand tile with the 128-byte swizzle (rows of
// 128 bytes, 8-row groups 1024 bytes apart): start address >> 4 (bits 0-13), leading offset 16
// bytes (unused by this layout), stride offset 1024 >> 4 (bits 32-45), descriptor version 1
// (bits 46-47), layout type 2 = 128-byte swizzle (bits 61-63).
__device__ __forceinline__ uint64_t sw128Desc(uint32_t saddr) {
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) |
           ((uint64_t)2 << 61);
}

__device__ __forceinline__ void mbarInit(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbarTryWait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the completion of phase `parity`; false when it gave up.
__device__ __forceinline__ bool mbarWait(uint32_t bar, uint32_t parity) {
    for (unsigned it = 0; it < kSpinLimit; it++)
        if (mbarTryWait(bar, parity)) return true;
    return false;
}
__device__ __forceinline__ void tmaLoad2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void fenceBefore() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfter() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void mmaBf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void mmaCommit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, uint32_t r[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float geluTanhF(float a) {
    const float c = 0.7978845608028654f, u = c * (a + 0.044715f * a * a * a);
    return 0.5f * a * (1.f + tanhf(u));
}

__global__ void __launch_bounds__(kGThreads, 1)
    k_umma_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int M, int N, int K,
                GemmEpilogue E) {
    extern __shared__ unsigned char smraw[];
    const uintptr_t base = (reinterpret_cast<uintptr_t>(smraw) + 1023) & ~uintptr_t(1023);  // swizzle atoms: 1 KB
    unsigned char *sA = reinterpret_cast<unsigned char *>(base);
    unsigned char *sB = sA + kGStages * kTileBytes;
    uint64_t *bars = reinterpret_cast<uint64_t *>(sB + kGStages * kTileBytes);  // full[S], empty[S], done
    uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(bars + 2 * kGStages + 1);
    __shared__ int sFail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // x runs over the column tiles: the CTAs that share a 128-row slice of A run together, so A is
    // read from DRAM about once (B, the smaller operand, stays in L2)
    const int m0 = blockIdx.y * kGM, n0 = blockIdx.x * kGN;
    const int kBlocks = K / kGK;
    auto full = [&](int s) { return sAddr(bars + s); };
    auto empty = [&](int s) { return sAddr(bars + kGStages + s); };
    const uint32_t done = sAddr(bars + 2 * kGStages);
    if (threadIdx.x == 0) {
        for (int s = 0; s < kGStages; s++) {
            mbarInit(full(s), 1);
            mbarInit(empty(s), 1);
        }
        mbarInit(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        sFail = 0;
    }
    if (warp == 0) {  // the whole warp allocates the accumulator's TMEM columns
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(sAddr(tmemSlot)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fenceBefore();
    __syncthreads();
    fenceAfter();
    const uint32_t tmem = *tmemSlot;
    int issued = 0;  // TMA stage loads issued by the producer
    if (warp == 0 && lane == 0) {
        for (int kb = 0; kb < kBlocks; kb++) {
            const int s = kb % kGStages, round = kb / kGStages;
            if (round > 0 && !mbarWait(empty(s), (round - 1) & 1)) {
                sFail = 1;
                atomicExch(E.err, 1);
                break;
            }
            mbarExpectTx(full(s), 2 * kTileBytes);
            tmaLoad2d(sAddr(sA + s * kTileBytes), &tmA, kb * kGK, m0, full(s));
            tmaLoad2d(sAddr(sB + s * kTileBytes), &tmB, kb * kGK, n0, full(s));
            issued++;
        }
    } else if (warp == 1 && lane == 0) {
        for (int kb = 0; kb < kBlocks; kb++) {
            const int s = kb % kGStages, round = kb / kGStages;
            if (!mbarWait(full(s), round & 1)) {
                sFail = 1;
                atomicExch(E.err, 2);
                break;
            }
            fenceAfter();
            const uint32_t a0 = sAddr(sA + s * kTileBytes), b0 = sAddr(sB + s * kTileBytes);
#pragma unroll
            for (int j = 0; j < kGK / 16; j++)  // K = 16 per instruction: 32 bytes along the swizzled rows
                mmaBf16(tmem, sw128Desc(a0 + 32 * j), sw128Desc(b0 + 32 * j), (kb | j) != 0);
            mmaCommit(empty(s));
        }
        mmaCommit(done);  // arrives once every MMA issued above has completed
    }
    __syncwarp();
    if (!mbarWait(done, 0)) {
        sFail = 1;
        atomicExch(E.err, 3);
    }
    __syncthreads();  // sFail is final: the epilogue's tcgen05.ld run in every warp or in none
    fenceAfter();
    if (!sFail) {
        const int row = m0 + warp * 32 + lane;
        const uint32_t tRow = tmem + ((uint32_t)(warp * 32) << 16);
        for (int c = 0; c < kGN; c += 16) {
            uint32_t r[16];
            tmemLoad16(tRow + c, r);
            if (row >= M) continue;
            const float ra = E.rowAdd ? E.rowAdd[row] : 0.f;
#pragma unroll
            for (int q = 0; q < 16; q++) {
                const int col = n0 + c + q;
                if (col >= N) break;
                float v = E.alpha * __uint_as_float(r[q]) + ra + (E.colAdd ? E.colAdd[col] : 0.f);
                if (E.D) E.D[(size_t)row * E.ldd + col] = v;
                if (E.D64) E.D64[(size_t)row * E.ldd + col] = (double)v;
                if (E.gelu) v = geluTanhF(v);
                if (E.Dact) E.Dact[(size_t)row * E.ldd + col] = v;
                if (E.Dbf) E.Dbf[(size_t)row * E.lddBf + col] = __float2bfloat16_rn(v);
            }
        }
    }
    if (warp == 0 && lane == 0)  // no copy of ours may still be writing this CTA's shared memory
        for (int kb = (issued > kGStages ? issued - kGStages : 0); kb < issued; kb++)
            if (!mbarWait(full(kb % kGStages), (kb / kGStages) & 1)) atomicExch(E.err, 4);
    fenceBefore();
    __syncthreads();
    if (warp == 0) {
        fenceAfter();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encodeFn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    if (!fn) throw std::runtime_error("[gemm] cuTensorMapEncodeTiled is not available");
    return fn;
}

// 2-D tensor map of a row-major BF16 matrix (rows x K), boxes of 128 rows x 64 columns, 128-byte
// swizzle; rows past the end read as zeros.
CUtensorMap tensorMap(const void *ptr, long rows, int K) {
    CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)K * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kGK, (cuuint32_t)kGM};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encodeFn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
                                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                  CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("[gemm] tensor map encoding failed (" + std::to_string((int)r) + ")");
    return m;
}

}  // namespace

void gemmBf16(const void *A, const void *B, long M, long N, int K, const GemmEpilogue &E, cudaStream_t stream) {
    if (M < 1 || N < 1 || K < kGK || K % kGK)
        throw std::invalid_argument("[gemm] sizes must be positive and K a multiple of 64");
    if (((uintptr_t)A | (uintptr_t)B) & 15) throw std::invalid_argument("[gemm] operands must be 16-byte aligned");
    if (M > 65535L * kGM || N > (1L << 30)) throw std::invalid_argument("[gemm] problem too large");
    if (!E.err) throw std::invalid_argument("[gemm] an error flag is required");
    static std::once_flag attr;
    std::call_once(attr, [] { cudaFuncSetAttribute(k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem); });
    const CUtensorMap ta = tensorMap(A, M, K), tb = tensorMap(B, N, K);
    const dim3 grid((unsigned)((N + kGN - 1) / kGN), (unsigned)((M + kGM - 1) / kGM));
    k_umma_gemm<<<grid, kGThreads, kGemmSmem, stream>>>(ta, tb, (int)M, (int)N, K, E);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) throw std::runtime_error(std::string("[gemm] launch: ") + cudaGetErrorString(e));
}

}  // namespace spock

namespace spock {
namespace {
int *errFlag(int device) {  // one device int per GPU for the stand-alone entry point
    static std::mutex mu;
    static int *flags[64] = {};
    if (device < 0 || device >= 64) throw std::invalid_argument("[gemm] device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!flags[device]) {
        cudaError_t e = cudaMalloc(&flags[device], sizeof(int));
        if (e != cudaSuccess) throw std::runtime_error(std::string("[gemm] cudaMalloc: ") + cudaGetErrorString(e));
    }
    return flags[device];
}
}  // namespace
}  // namespace spock

extern "C" int spock_gemm_bf16(const void *A, const void *B, long M, long N, int K, float alpha, const float *rowAdd,
                               const float *colAdd, int gelu, float *D, float *Dact, long ldd, int device) {
    return spock::guardedCall([&] {
        if (!A || !B || (!D && !Dact)) throw std::invalid_argument("[gemm] null device pointer");
        if (ldd < N) throw std::invalid_argument("[gemm] ldd < N");
        cudaError_t e = cudaSetDevice(device);
        if (e != cudaSuccess) throw std::runtime_error(std::string("[gemm] cudaSetDevice: ") + cudaGetErrorString(e));
        int *err = spock::errFlag(device);
        if ((e = cudaMemset(err, 0, sizeof(int))) != cudaSuccess)
            throw std::runtime_error(std::string("[gemm] ") + cudaGetErrorString(e));
        spock::GemmEpilogue E;
        E.alpha = alpha;
        E.rowAdd = rowAdd;
        E.colAdd = colAdd;
        E.gelu = gelu;
        E.D = D;
        E.Dact = Dact;
        E.ldd = ldd;
        E.err = err;
        spock::gemmBf16(A, B, M, N, K, E, nullptr);
        int h = 0;
        if ((e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
            throw std::runtime_error(std::string("[gemm] ") + cudaGetErrorString(e));
        if (h) throw std::runtime_error("[gemm] the tensor-core pipeline gave up (code " + std::to_string(h) + ")");
    });
}

extern "C" int spock_warm_start_pca(spock_solver s, const void *basis, const void *coef, int k, const float *mean) {
    return spock::guardedCall([&] {
        spock::EngineBase *eng = spock::engineOf(s);
        cudaError_t e = cudaSetDevice(eng->device());
        if (e != cudaSuccess) throw std::runtime_error(std::string("[warmStart] cudaSetDevice: ") + cudaGetErrorString(e));
        eng->warmStartPca(basis, coef, k, mean);
    });
}
