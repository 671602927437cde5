// One instantiation of the batched L* or L kernel with its host launcher.  build.py compiles this
// file once per kernel (SPOCK_OPS_LSTAR or SPOCK_OPS_LOP), precision (SPOCK_OPS_T) and mode
// (SPOCK_OPS_MODE); the twelve objects compile in parallel.
#include "kernels_batch.cuh"

#if !defined(SPOCK_OPS_T) || !defined(SPOCK_OPS_MODE)
#error "ops_batch.cu needs SPOCK_OPS_T and SPOCK_OPS_MODE"
#endif

namespace spock {

#if defined(SPOCK_OPS_LSTAR)
template <typename T, int MODE>
void launchLstarB(dim3 grid, size_t smem, cudaStream_t stream, const DevProblem<T> &P, const Dims &D, const OpArgs<T> &A,
                  const PadMats<T> &M, int tilesPerCta, int dbl) {
    k_lstar_b<T, MODE><<<grid, kTileB * kTileWarps, smem, stream>>>(P, D, A, M, tilesPerCta, dbl);
}
template <typename T, int MODE>
cudaError_t optInLstarB(int bytes) {
    return cudaFuncSetAttribute(k_lstar_b<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
template void launchLstarB<SPOCK_OPS_T, SPOCK_OPS_MODE>(dim3, size_t, cudaStream_t, const DevProblem<SPOCK_OPS_T> &,
                                                        const Dims &, const OpArgs<SPOCK_OPS_T> &,
                                                        const PadMats<SPOCK_OPS_T> &, int, int);
template cudaError_t optInLstarB<SPOCK_OPS_T, SPOCK_OPS_MODE>(int);
#elif defined(SPOCK_OPS_LOP)
template <typename T, int MODE>
void launchLopB(dim3 grid, size_t smem, cudaStream_t stream, const DevProblem<T> &P, const Dims &D, const OpArgs<T> &A,
                const PadMats<T> &M, int tilesPerCta, int dbl) {
    k_lop_b<T, MODE><<<grid, kTileB * kTileWarps, smem, stream>>>(P, D, A, M, tilesPerCta, dbl);
}
template <typename T, int MODE>
cudaError_t optInLopB(int bytes) {
    return cudaFuncSetAttribute(k_lop_b<T, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}
template void launchLopB<SPOCK_OPS_T, SPOCK_OPS_MODE>(dim3, size_t, cudaStream_t, const DevProblem<SPOCK_OPS_T> &,
                                                      const Dims &, const OpArgs<SPOCK_OPS_T> &,
                                                      const PadMats<SPOCK_OPS_T> &, int, int);
template cudaError_t optInLopB<SPOCK_OPS_T, SPOCK_OPS_MODE>(int);
#else
#error "ops_batch.cu needs SPOCK_OPS_LSTAR or SPOCK_OPS_LOP"
#endif

}  // namespace spock
