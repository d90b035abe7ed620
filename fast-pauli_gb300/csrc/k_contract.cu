// k_contract.cu -- the SummedPauliOp coefficient contractions on CUDA cores.
//
//  * launch_contract_real: out(K,S) += H^T E, H complex (P,K), E real (P,S):
//    the contraction of SummedPauliOp::expectation_value
//    (fast_pauli/cpp/include/__summed_pauli_op.hpp:579-591), with real E
//    because per-string expectation values of Hermitian Pauli strings are real
//    (so two real GEMMs instead of a complex one).
//  * launch_weighted_coeffs: W(P,S) = H X, X real (K,S): the weighted
//    coefficients of SummedPauliOp::apply_weighted (__summed_pauli_op.hpp:420-432).
//
// Float64 arithmetic (the plain form).  64x64 output tiles, 16-deep k steps
// staged in shared memory, 4x4 outputs per thread.
#include "common.cuh"

namespace fpg
{
namespace
{

constexpr int BM = 64, BN = 64, BK = 16;

template <typename HC> struct HT; // complex element type of H
template <> struct HT<double2>
{
    __device__ static double2 ld(const void *p, int64_t i)
    {
        return reinterpret_cast<const double2 *>(p)[i];
    }
};
template <> struct HT<float2>
{
    __device__ static double2 ld(const void *p, int64_t i)
    {
        const float2 f = reinterpret_cast<const float2 *>(p)[i];
        return make_double2(f.x, f.y);
    }
};

// C(M,N) (+)= A(M,Kd) B(Kd,N); A complex, B real, C complex.
// A_T: A(m,p) stored as Hs[p * lda + m] (transposed), else Hs[m * lda + p].
// only_if: when not null, return at once unless *only_if is set (the float64
// form behind the tensor-core contraction, for non-finite inputs).
template <typename HC, typename BR, typename OC, bool A_T, bool ACCUM>
__global__ void __launch_bounds__(256)
    k_gemm_cr(const void *__restrict__ Araw, int64_t lda, const BR *__restrict__ B, int64_t M, int64_t N, int64_t Kd,
              OC *__restrict__ C, const int *__restrict__ only_if)
{
    if (only_if && *only_if == 0)
        return;
    __shared__ double As_r[BK][BM];
    __shared__ double As_i[BK][BM];
    __shared__ double Bs[BK][BN];
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
    double cr[4][4], ci[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            cr[i][j] = ci[i][j] = 0.0;

    for (int64_t p0 = 0; p0 < Kd; p0 += BK)
    {
        // A tile: BK x BM complex
        for (int e = tid; e < BK * BM; e += 256)
        {
            int kk, mm;
            if (A_T)
            {
                kk = e / BM;
                mm = e % BM;
            }
            else
            {
                mm = e / BK;
                kk = e % BK;
            }
            const int64_t p = p0 + kk, m = m0 + mm;
            double2 a = make_double2(0.0, 0.0);
            if (p < Kd && m < M)
                a = HT<HC>::ld(Araw, A_T ? p * lda + m : m * lda + p);
            As_r[kk][mm] = a.x;
            As_i[kk][mm] = a.y;
        }
        for (int e = tid; e < BK * BN; e += 256)
        {
            const int kk = e / BN, nn = e % BN;
            const int64_t p = p0 + kk, c = n0 + nn;
            Bs[kk][nn] = (p < Kd && c < N) ? (double)B[p * N + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk)
        {
            double ar[4], ai[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
            {
                ar[i] = As_r[kk][ty + 16 * i];
                ai[i] = As_i[kk][ty + 16 * i];
            }
#pragma unroll
            for (int j = 0; j < 4; ++j)
                b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j)
                {
                    cr[i][j] = fma(ar[i], b[j], cr[i][j]);
                    ci[i][j] = fma(ai[i], b[j], ci[i][j]);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
    {
        const int64_t m = m0 + ty + 16 * i;
        if (m >= M)
            continue;
#pragma unroll
        for (int j = 0; j < 4; ++j)
        {
            const int64_t c = n0 + tx + 16 * j;
            if (c >= N)
                continue;
            OC &dst = C[m * N + c];
            if (ACCUM)
            {
                dst.x += cr[i][j];
                dst.y += ci[i][j];
            }
            else
            {
                dst.x = cr[i][j];
                dst.y = ci[i][j];
            }
        }
    }
}

} // namespace

cudaError_t launch_contract_real(bool out_c64, const void *H, bool h_c64, const double *E, int64_t P, int64_t K,
                                 int64_t S, void *out, cudaStream_t st)
{
    if (K <= 0 || S <= 0)
        return cudaSuccess;
    dim3 grid((unsigned)((S + BN - 1) / BN), (unsigned)((K + BM - 1) / BM));
    if (!out_c64 && !h_c64)
        k_gemm_cr<double2, double, double2, true, true><<<grid, 256, 0, st>>>(H, K, E, K, S, P, (double2 *)out, nullptr);
    else if (out_c64 && h_c64)
        k_gemm_cr<float2, double, float2, true, true><<<grid, 256, 0, st>>>(H, K, E, K, S, P, (float2 *)out, nullptr);
    else if (out_c64)
        k_gemm_cr<double2, double, float2, true, true><<<grid, 256, 0, st>>>(H, K, E, K, S, P, (float2 *)out, nullptr);
    else
        k_gemm_cr<float2, double, double2, true, true><<<grid, 256, 0, st>>>(H, K, E, K, S, P, (double2 *)out, nullptr);
    return launched();
}

cudaError_t launch_contract_f64_if(const void *H, const double *E, int64_t P, int64_t K, int64_t S, void *out,
                                   const int *only_if, cudaStream_t st)
{
    if (K <= 0 || S <= 0)
        return cudaSuccess;
    dim3 grid((unsigned)((S + BN - 1) / BN), (unsigned)((K + BM - 1) / BM));
    k_gemm_cr<double2, double, double2, true, true>
        <<<grid, 256, 0, st>>>(H, K, E, K, S, P, (double2 *)out, only_if);
    return launched();
}

cudaError_t launch_weighted_coeffs(bool fp32, const void *H, const void *X, int64_t P, int64_t K, int64_t S, void *W,
                                   cudaStream_t st)
{
    if (P <= 0 || S <= 0)
        return cudaSuccess;
    dim3 grid((unsigned)((S + BN - 1) / BN), (unsigned)((P + BM - 1) / BM));
    if (!fp32)
        k_gemm_cr<double2, double, double2, false, false>
            <<<grid, 256, 0, st>>>(H, K, (const double *)X, P, S, K, (double2 *)W, nullptr);
    else
        k_gemm_cr<float2, float, float2, false, false>
            <<<grid, 256, 0, st>>>(H, K, (const float *)X, P, S, K, (float2 *)W, nullptr);
    return launched();
}

} // namespace fpg
