// k_expect_marg.cu -- per-string expectation values for x-groups whose
// strings each have a sign pattern of one row bit at most.
//
// Same quantity as k_expect.cu (the per-string stage of
// SummedPauliOp::expectation_value, fast_pauli/cpp/include/__summed_pauli_op.hpp:572-577).
// With the pairing bit p (top bit of x) dropped, every string of such a group
// has z' = 0 or z' = e_b for some row bit b (e.g. the 2 + 2(n-1) strings
// X_a, Y_a, X_a Z_b, Y_a Z_b of a weight <= 2 set share x = e_a).  Then
//     sum_i (-1)^popc(i & z') v(i) = T            (z' = 0)
//                                  = T - 2 M_b    (z' = e_b),
// T = sum_i v(i), M_b = sum_{i: bit b of i set} v(i), so the whole group needs
// only the total and one "marginal" per row bit -- for Re q and Im q -- not a
// sum per string.  Per 32-row block the marginals of the five low bits come
// from a small tree (4-row groups: pair sums, then group sums), ~2.1 adds per
// row and part; the block total is added to the marginal of each higher bit
// set in the block's base.  Per row that is q (4 operations) plus ~4.3 adds
// for both parts, against ~14 for the 16-point transform kernel.
//
// Rows: as k_expect_pair.cu -- blocks paired for x >= 32, rows paired inside
// a block for 0 < x < 32 (16 rows visited), all rows for x = 0.  Layout: TC
// column lanes x (256 / TC) row lanes, one complex element per lane; grid
// (chunks, row splits, column tiles).  float32 path: block sums in float32,
// Kahan-compensated across blocks; float64 across threads.
#include "expect_body.cuh"

namespace fpg
{
namespace
{

template <typename T> __device__ __forceinline__ void kadd(T &acc, T &cmp, T x)
{
    if constexpr (sizeof(T) == 8)
    {
        acc += x;
    }
    else
    {
        const T y = x - cmp;
        const T s = acc + y;
        cmp = (s - acc) - y;
        acc = s;
    }
}

template <typename T> struct Cplx;
template <> struct Cplx<double>
{
    using type = double2;
};
template <> struct Cplx<float>
{
    using type = float2;
};

// Sums of one block: bt[part] (total) and bl[part][j] (rows whose visited-row
// bit j is set).  LB = 5: all 32 rows, visited bit j = row bit j.  LB = 4:
// the 16 rows with bit pl clear; visited bit j = row bit (j < pl ? j : j + 1).
template <typename T, int LB>
__device__ __forceinline__ void block_marginals(const T *__restrict__ psi, int64_t S, int64_t t0, uint64_t base,
                                                uint64_t baseB, uint32_t xl, int pl, int RB, bool need_re,
                                                bool need_im, T (&bt)[2], T (&bl)[2][5])
{
    using CT = typename Cplx<T>::type;
    const CT *ps = reinterpret_cast<const CT *>(psi);
    // 16 visited rows at a time (LB = 5: two halves, bit 4 from the half)
#pragma unroll 1
    for (int h = 0; h < (1 << (LB - 4)); ++h)
    {
        T hs[2] = {T(0), T(0)};
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            T v[4][2];
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                const uint32_t m2 = (uint32_t)(16 * h + 4 * k + u);
                const uint32_t r = LB == 5 ? m2 : (((m2 >> pl) << (pl + 1)) | (m2 & ((1u << pl) - 1u)));
                v[u][0] = T(0);
                v[u][1] = T(0);
                if ((int)r < RB)
                {
                    const CT a = __ldg(ps + (int64_t)(base + r) * S + t0);
                    const CT b = __ldg(ps + (int64_t)(baseB + (uint64_t)(r ^ xl)) * S + t0);
                    if (need_re)
                        v[u][0] = fma(a.x, b.x, a.y * b.y);
                    if (need_im)
                        v[u][1] = fma(a.x, b.y, -(a.y * b.x));
                }
            }
#pragma unroll
            for (int p = 0; p < 2; ++p)
            {
                if (p == 0 ? !need_re : !need_im)
                    continue;
                const T p0 = v[0][p] + v[1][p];
                const T p1 = v[2][p] + v[3][p];
                bl[p][0] += v[1][p];
                bl[p][0] += v[3][p];
                bl[p][1] += p1;
                const T g = p0 + p1;
                hs[p] += g;
                if (k & 1)
                    bl[p][2] += g;
                if (k & 2)
                    bl[p][3] += g;
            }
        }
#pragma unroll
        for (int p = 0; p < 2; ++p)
        {
            bt[p] += hs[p];
            if (h)
                bl[p][4] += hs[p];
        }
    }
}

template <typename T> constexpr int kMargMinBlocks = 2;

template <typename T, int NH>
__global__ void __launch_bounds__(256, kMargMinBlocks<T>)
    k_expect_marg(const T *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                  const int32_t *__restrict__ orig, int64_t P, const MargChunk *__restrict__ chunks, int TC,
                  int n_splits, double *__restrict__ out)
{
    constexpr int NV = 2 * (1 + 5 + NH); // values per thread: [part][total, low 5, high NH]
    constexpr int NVB = 8;               // values reduced per pass
    extern __shared__ double smem[];
    double *red = smem;                  // [NVB][256]
    double *res = smem + NVB * 256;      // [NV][TC] totals per column lane

    const MargChunk ch = chunks[blockIdx.x];
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const int64_t t0 = (int64_t)blockIdx.z * TC + tc;
    const bool col_ok = t0 < S;

    const uint64_t D = 1ull << n;
    const uint64_t xh = ch.x & ~31ull;
    const uint32_t xl = (uint32_t)ch.x & 31u;
    const bool paired = xh != 0;
    const int pl = (!paired && xl != 0u) ? (31 - __clz((int)xl)) : -1;
    const int64_t NB = n >= 5 ? (int64_t)(D >> 5) : 1;
    const int RB = n >= 5 ? 32 : (int)D;
    const int64_t nblk = paired ? NB / 2 : NB;
    const int hb = paired ? (63 - __clzll((long long)(xh >> 5))) : 0;
    const int64_t per = (nblk + n_splits - 1) / n_splits;
    const int64_t b0 = (int64_t)blockIdx.y * per;
    const int64_t b1 = min(nblk, b0 + per);
    const bool need_re = (ch.flags & 1) != 0, need_im = (ch.flags & 2) != 0;

    // row bits >= 5 used by the strings (at most NH; unused slots -> bit 63,
    // never set in a row index)
    int hpos[NH];
    {
        uint64_t hm = ch.zmask & ~31ull;
#pragma unroll
        for (int j = 0; j < NH; ++j)
        {
            hpos[j] = hm ? (__ffsll((long long)hm) - 1) : 63;
            hm &= hm - 1ull;
        }
    }

    T tot[2], totc[2], ml[2][5], mlc[2][5], mh[2][NH], mhc[2][NH];
#pragma unroll
    for (int p = 0; p < 2; ++p)
    {
        tot[p] = totc[p] = T(0);
#pragma unroll
        for (int j = 0; j < 5; ++j)
            ml[p][j] = mlc[p][j] = T(0);
#pragma unroll
        for (int j = 0; j < NH; ++j)
            mh[p][j] = mhc[p][j] = T(0);
    }

    if (col_ok)
    {
        for (int64_t m = b0 + tr; m < b1; m += TR)
        {
            const uint64_t um = (uint64_t)m;
            const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
            const uint64_t base = beta << 5;
            const uint64_t baseB = base ^ xh;
            T bt[2] = {T(0), T(0)};
            T bl[2][5];
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int j = 0; j < 5; ++j)
                    bl[p][j] = T(0);
            if (pl < 0)
                block_marginals<T, 5>(psi, S, t0, base, baseB, xl, pl, RB, need_re, need_im, bt, bl);
            else
                block_marginals<T, 4>(psi, S, t0, base, baseB, xl, pl, RB, need_re, need_im, bt, bl);
#pragma unroll
            for (int p = 0; p < 2; ++p)
            {
                kadd(tot[p], totc[p], bt[p]);
#pragma unroll
                for (int j = 0; j < 5; ++j)
                    kadd(ml[p][j], mlc[p][j], bl[p][j]);
#pragma unroll
                for (int j = 0; j < NH; ++j)
                    if ((base >> hpos[j]) & 1ull)
                        kadd(mh[p][j], mhc[p][j], bt[p]);
            }
        }
    }

    // deterministic float64 reduction over the row lanes, NVB values a pass
#pragma unroll
    for (int v0 = 0; v0 < NV; v0 += NVB)
    {
#pragma unroll
        for (int w = 0; w < NVB; ++w)
        {
            const int v = v0 + w;
            if (v < NV)
            {
                const int p = v / (NV / 2), i = v % (NV / 2);
                double x;
                if (i == 0)
                    x = (double)tot[p] - (double)totc[p];
                else if (i < 6)
                    x = (double)ml[p][i - 1] - (double)mlc[p][i - 1];
                else
                    x = (double)mh[p][i - 6] - (double)mhc[p][i - 6];
                red[w * 256 + tid] = x;
            }
        }
        __syncthreads();
        for (int s = TR >> 1; s > 0; s >>= 1)
        {
            if (tr < s)
#pragma unroll
                for (int w = 0; w < NVB; ++w)
                    red[w * 256 + tid] += red[w * 256 + tid + s * TC];
            __syncthreads();
        }
        if (tr == 0)
#pragma unroll
            for (int w = 0; w < NVB; ++w)
                if (v0 + w < NV)
                    res[(v0 + w) * TC + tc] = red[w * 256 + tc];
        __syncthreads();
    }
    if (!col_ok)
        return;

    // every string: f * (T - 2 M_b) or f * T; row lanes share the strings
    const uint64_t pbit = paired ? (1ull << (hb + 5)) : (pl >= 0 ? (1ull << pl) : 0ull);
    const uint64_t hmask = ch.zmask & ~31ull;
    for (int k = tr; k < ch.count; k += TR)
    {
        const int sidx = ch.begin + k;
        const StringRec rec = recs[sidx];
        const int p = (int)(rec.meta & 1u);
        const uint64_t zp = rec.z & ~pbit;
        double val = res[(p * (NV / 2)) * TC + tc];
        if (zp)
        {
            const int b = __ffsll((long long)zp) - 1;
            int i;
            if (b < 5)
                i = 1 + ((pl >= 0 && b > pl) ? b - 1 : b);
            else
                i = 6 + __popcll(hmask & ((1ull << b) - 1ull));
            val -= 2.0 * res[(p * (NV / 2) + i) * TC + tc];
        }
        const int ny = (int)(rec.meta & 3u);
        const double f = ((ny & 2) ? -1.0 : 1.0) * (pbit ? 2.0 : 1.0);
        out[((int64_t)blockIdx.y * P + orig[sidx]) * S + t0] = f * val;
    }
}

template <typename T, int NH>
void launch_nh(const T *psi, int64_t S, int n, const DevOp &op, const MargChunk *d_chunks, int n_chunks, int TC,
               int n_ctiles, int n_splits, double *out, cudaStream_t st)
{
    constexpr int NV = 2 * (1 + 5 + NH);
    const size_t smem = (size_t)(8 * 256 + NV * TC) * sizeof(double);
    dim3 grid((unsigned)n_chunks, (unsigned)n_splits, (unsigned)n_ctiles);
    k_expect_marg<T, NH><<<grid, 256, smem, st>>>(psi, S, n, op.recs, op.orig, op.P, d_chunks, TC, n_splits, out);
}

} // namespace

cudaError_t launch_expect_marg(bool fp32, const void *psi, int64_t S, int n, const DevOp &op,
                               const MargChunk *d_chunks, int n_chunks, int max_high_bits, int TC, int n_ctiles,
                               int n_splits, double *out, cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    if (max_high_bits > kMargMaxHighBits)
        return cudaErrorInvalidValue;
#define FPG_MARG(NH)                                                                                                   \
    if (fp32)                                                                                                          \
        launch_nh<float, NH>((const float *)psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, st);     \
    else                                                                                                               \
        launch_nh<double, NH>((const double *)psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, st);
    if (max_high_bits <= 9)
    {
        FPG_MARG(9)
    }
    else
    {
        FPG_MARG(18)
    }
#undef FPG_MARG
    return launched();
}

} // namespace fpg
