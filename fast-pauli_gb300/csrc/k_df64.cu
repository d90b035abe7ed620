// k_df64.cu -- the float64 state as df64 pairs, once per call.
//
// The float64 expectation kernels run in double-float arithmetic on the
// float32 pipes (df64.cuh).  Every amplitude is read by many x-groups (91
// times per launch for the weight-2 pairs of a 14-qubit operator), so
// splitting it into (hi, lo) floats once, into a scratch copy of the same
// size, takes the integer split work out of their inner loops.  The pass
// also raises the call's range flag for amplitudes outside the df64 range,
// after which the float64 kernels recompute the result.
#include "common.cuh"
#include "df64.cuh"

namespace fpg
{
namespace
{

__global__ void __launch_bounds__(256) k_df_split(const uint4 *__restrict__ psi, int64_t count, float4 *__restrict__ out,
                                                  int *__restrict__ range_flag)
{
    bool bad = false;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = split_complex(__ldg(psi + i), bad);
    if (__syncthreads_or(bad) && threadIdx.x == 0)
        atomicOr(range_flag, 1);
}

} // namespace

cudaError_t launch_df_split(const void *psi, int64_t count, void *out, int *range_flag, cudaStream_t st)
{
    if (count <= 0)
        return cudaSuccess;
    int64_t blocks = (count + 255) / 256;
    if (blocks > (int64_t)sm_count() * 16)
        blocks = (int64_t)sm_count() * 16;
    k_df_split<<<(unsigned)blocks, 256, 0, st>>>((const uint4 *)psi, count, (float4 *)out, range_flag);
    return launched();
}

} // namespace fpg
