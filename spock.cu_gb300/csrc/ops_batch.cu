// One instantiation of the batched L* or L kernel with its host launcher.  build.py compiles this
// file once per kernel (SPOCK_OPS_LSTAR or SPOCK_OPS_LOP), precision (SPOCK_OPS_T), mode
// (SPOCK_OPS_MODE) and matrix placement (SPOCK_OPS_GM: 1 reads node matrices in place); the
// objects compile in parallel.
#include "kernels_batch.cuh"

#if !defined(SPOCK_OPS_T) || !defined(SPOCK_OPS_MODE) || !defined(SPOCK_OPS_GM)
#error "ops_batch.cu needs SPOCK_OPS_T, SPOCK_OPS_MODE and SPOCK_OPS_GM"
#endif

namespace spock {

#if defined(SPOCK_OPS_LSTAR)
template <typename T, int MODE, bool GM>
void launchLstarB(dim3 grid, size_t smem, cudaStream_t stream, const DevProblem<T> &P, const Dims &D, const OpArgs<T> &A,
                  const PadMats<T> &M, int tilesPerCta, int dbl) {
    k_lstar_b<T, MODE, GM><<<grid, kTileB * kTileWarps, smem, stream>>>(P, D, A, M, tilesPerCta, dbl);
}
template <typename T, int MODE, bool GM>
cudaError_t optInLstarB(int bytes) {
    return cudaFuncSetAttribute(k_lstar_b<T, MODE, GM>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
template void launchLstarB<SPOCK_OPS_T, SPOCK_OPS_MODE, (SPOCK_OPS_GM != 0)>(dim3, size_t, cudaStream_t, const DevProblem<SPOCK_OPS_T> &,
                                                        const Dims &, const OpArgs<SPOCK_OPS_T> &,
                                                        const PadMats<SPOCK_OPS_T> &, int, int);
template cudaError_t optInLstarB<SPOCK_OPS_T, SPOCK_OPS_MODE, (SPOCK_OPS_GM != 0)>(int);
#elif defined(SPOCK_OPS_LOP)
template <typename T, int MODE, bool GM>
void launchLopB(dim3 grid, size_t smem, cudaStream_t stream, const DevProblem<T> &P, const Dims &D, const OpArgs<T> &A,
                const PadMats<T> &M, int tilesPerCta, int dbl) {
    k_lop_b<T, MODE, GM><<<grid, kTileB * kTileWarps, smem, stream>>>(P, D, A, M, tilesPerCta, dbl);
}
template <typename T, int MODE, bool GM>
cudaError_t optInLopB(int bytes) {
    return cudaFuncSetAttribute(k_lop_b<T, MODE, GM>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
template void launchLopB<SPOCK_OPS_T, SPOCK_OPS_MODE, (SPOCK_OPS_GM != 0)>(dim3, size_t, cudaStream_t, const DevProblem<SPOCK_OPS_T> &,
                                                      const Dims &, const OpArgs<SPOCK_OPS_T> &,
                                                      const PadMats<SPOCK_OPS_T> &, int, int);
template cudaError_t optInLopB<SPOCK_OPS_T, SPOCK_OPS_MODE, (SPOCK_OPS_GM != 0)>(int);
#else
#error "ops_batch.cu needs SPOCK_OPS_LSTAR or SPOCK_OPS_LOP"
#endif

}  // namespace spock
