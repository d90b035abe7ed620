// k_df64.cu -- the float64 state as df64 pairs, once per call.
//
// The float64 expectation kernels run in double-float arithmetic on the
// float32 pipes (df64.cuh).  Every amplitude is read by many x-groups (91
// times per launch for the weight-2 pairs of a 14-qubit operator), so
// splitting it into (hi, lo) floats once, into a scratch copy of the same
// size, takes the integer split work out of their inner loops.  The pass
// also raises the call's range flag for amplitudes and columns outside the
// df64 range (df64.cuh), after which the float64 kernels recompute the
// result.
#include <algorithm>

#include "common.cuh"
#include "df64.cuh"

namespace fpg
{
namespace
{

// rows x cols complex128 elements, row-major.  Thread (cl, rl) of a CTA
// covers column blockIdx.x * TCc + cl and rows blockIdx.y * R + rl + k R
// gridDim.y (TCc = min(cols, 256) columns, R = 256 / TCc rows per pass), so
// a warp reads consecutive elements and a thread keeps one column: its
// largest high word of |x| goes to colmax once.  out == nullptr: the check
// only (states too large for a split copy).
__global__ void __launch_bounds__(256) k_df_split(const uint4 *__restrict__ psi, int64_t rows, int64_t cols, int TCc,
                                                  float4 *__restrict__ out, uint32_t *__restrict__ colmax,
                                                  int *__restrict__ range_flag)
{
    bool bad = false;
    const int R = 256 / TCc;
    const int cl = (int)threadIdx.x % TCc, rl = (int)threadIdx.x / TCc;
    const int64_t c = (int64_t)blockIdx.x * TCc + cl;
    uint32_t key = 0;
    if (rl < R && c < cols)
    {
        const int64_t step = (int64_t)R * gridDim.y;
        for (int64_t r = (int64_t)blockIdx.y * R + rl; r < rows; r += step)
        {
            const uint4 w = __ldg(psi + r * cols + c);
            key = max(key, max(w.y & 0x7fffffffu, w.w & 0x7fffffffu));
            if (out)
                out[r * cols + c] = split_complex(w, bad);
            else
                bad |= df_out_of_range(w.y) | df_out_of_range(w.w);
        }
        if (key)
            atomicMax(colmax + c, key);
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0)
        atomicOr(range_flag, 1);
}

// a non-zero column whose largest |x| is below the df64 column bound
__global__ void k_df_columns(const uint32_t *__restrict__ colmax, int64_t cols, int *__restrict__ range_flag)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c < cols && colmax[c] != 0u && colmax[c] < kDfColumnMinKey)
        atomicOr(range_flag, 1);
}

} // namespace

size_t df_split_colmax_bytes(int64_t cols)
{
    return ((size_t)cols * sizeof(uint32_t) + 255) / 256 * 256;
}

cudaError_t launch_df_split(const void *psi, int64_t rows, int64_t cols, void *out, void *colmax, int *range_flag,
                            cudaStream_t st)
{
    if (rows <= 0 || cols <= 0)
        return cudaSuccess;
    if (cudaError_t e = cudaMemsetAsync(colmax, 0, (size_t)cols * sizeof(uint32_t), st))
        return e;
    const int TCc = cols < 256 ? (int)cols : 256;
    const int R = 256 / TCc;
    const int64_t gx = (cols + TCc - 1) / TCc;
    const int64_t want = (int64_t)sm_count() * 16;
    int64_t gy = std::max<int64_t>(1, want / gx);
    gy = std::min<int64_t>(gy, (rows + R - 1) / R);
    gy = std::min<int64_t>(gy, 65535);
    if (gx > 0x7fffffff)
        return cudaErrorInvalidValue;
    k_df_split<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, st>>>((const uint4 *)psi, rows, cols, TCc, (float4 *)out,
                                                                (uint32_t *)colmax, range_flag);
    if (cudaError_t e = launched())
        return e;
    k_df_columns<<<(unsigned)((cols + 255) / 256), 256, 0, st>>>((const uint32_t *)colmax, cols, range_flag);
    return launched();
}

} // namespace fpg
