// expect_body.cuh -- the per-chunk body of the expectation kernels, shared by
// the per-call kernel (k_expect.cu) and the persistent batch kernel
// (batch.cu).  See k_expect.cu for the algorithm.
#pragma once

#include "common.cuh"

namespace fpg
{

template <typename T, int V> struct Cvec; // V complex elements = 2V reals, one vector load
template <> struct Cvec<double, 1>
{
    using type = double2;
};
template <> struct Cvec<float, 1>
{
    using type = float2;
};
template <> struct Cvec<float, 2>
{
    using type = float4;
};

template <typename T, int V>
__device__ __forceinline__ void load_cvec(const T *p, T (&re)[V], T (&im)[V])
{
    using L = typename Cvec<T, V>::type;
    const L v = __ldg(reinterpret_cast<const L *>(p));
    if constexpr (V == 1)
    {
        re[0] = v.x;
        im[0] = v.y;
    }
    else
    {
        re[0] = v.x;
        im[0] = v.y;
        re[1] = v.z;
        im[1] = v.w;
    }
}

__device__ __forceinline__ float flip_sign(float v, uint32_t mask, int r)
{
    return __int_as_float(__float_as_int(v) ^ ((mask << (31 - r)) & 0x80000000u));
}
__device__ __forceinline__ double flip_sign(double v, uint32_t mask, int r)
{
    const int hi = __double2hiint(v) ^ (int)((mask << (31 - r)) & 0x80000000u);
    return __hiloint2double(hi, __double2loint(v));
}

// One chunk (<= GE even-#Y and <= GO odd-#Y strings of one x-group) over the
// column tile `ctile` and row split `split` of `n_splits`.  All threads of the
// CTA call it with the same arguments.  Results (f * sum, float64) go to
// out[(split * P + orig) * S + t].  red: blockDim.x * V doubles of shared memory.
template <typename T, int V, int GE, int GO>
__device__ __forceinline__ void expect_chunk_body(const T *__restrict__ psi, int64_t S, int n,
                                                  const StringRec *__restrict__ recs,
                                                  const int32_t *__restrict__ orig, int64_t P, const Chunk ch, int TC,
                                                  int64_t ctile, int split, int n_splits, double *__restrict__ out,
                                                  double *red)
{
    constexpr int G = GE + GO;
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const int64_t t0 = (ctile * TC + tc) * V;
    const bool col_ok = t0 < S; // V == 2 only when S is even

    const uint64_t D = 1ull << n;
    const uint64_t xh = ch.x & ~31ull;
    const uint32_t xl = (uint32_t)ch.x & 31u;
    const bool paired = xh != 0;
    const int64_t NB = n >= 5 ? (int64_t)(D >> 5) : 1;
    const int RB = n >= 5 ? 32 : (int)D;
    const int64_t nblk = paired ? NB / 2 : NB;
    const int hb = paired ? (63 - __clzll((long long)(xh >> 5))) : 0;
    const int64_t per = (nblk + n_splits - 1) / n_splits;
    const int64_t b0 = (int64_t)split * per;
    const int64_t b1 = min(nblk, b0 + per);
    const int ne = ch.n_even, no = ch.n_odd;

    uint64_t z[G];
    uint32_t ml[G];
#pragma unroll
    for (int k = 0; k < GE; ++k)
    {
        const bool ok = k < ne;
        z[k] = ok ? recs[ch.begin_even + k].z : 0ull;
        ml[k] = ok ? recs[ch.begin_even + k].mask_lo : 0u;
    }
#pragma unroll
    for (int k = 0; k < GO; ++k)
    {
        const bool ok = k < no;
        z[GE + k] = ok ? recs[ch.begin_odd + k].z : 0ull;
        ml[GE + k] = ok ? recs[ch.begin_odd + k].mask_lo : 0u;
    }

    // accumulators: float64 path accumulates block sums directly; float32
    // path keeps a Kahan pair across blocks.
    T acc[G][V];
    T cmp[G][V];
#pragma unroll
    for (int k = 0; k < G; ++k)
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            acc[k][v] = T(0);
            cmp[k][v] = T(0);
        }

    if (col_ok)
    {
        for (int64_t m = b0 + tr; m < b1; m += TR)
        {
            const uint64_t um = (uint64_t)m;
            const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
            const uint64_t base = beta << 5;
            const uint64_t baseB = base ^ xh;
            uint32_t mk[G];
#pragma unroll
            for (int k = 0; k < G; ++k)
                mk[k] = ml[k] ^ (0u - (uint32_t)(__popcll(base & z[k]) & 1));

            T bs[G][V];
#pragma unroll
            for (int k = 0; k < G; ++k)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    bs[k][v] = T(0);

            const T *pa0 = psi + 2 * ((int64_t)base * S + t0);
            // rows in groups of RG: all loads of a group are issued before any
            // is consumed.  Single-string float32 chunks (random strings) have
            // almost no arithmetic per row and are bound by load latency: they
            // batch as many rows as fit the three-CTA register budget without
            // spilling (8 rows of one-column lanes, 5 of two-column lanes);
            // every other class keeps its registers for occupancy (measured:
            // deeper batches cost the weight-2 float32 classes a CTA per SM).
            constexpr int RG = (sizeof(T) == 4 && G == 1) ? (V == 1 ? 8 : 5) : 1;
#pragma unroll
            for (int r0 = 0; r0 < 32; r0 += RG)
            {
                T ar[RG][V], ai[RG][V], br[RG][V], bi[RG][V];
#pragma unroll
                for (int g = 0; g < RG; ++g)
                {
                    const int r = r0 + g;
                    if (r < RB)
                    {
                        load_cvec<T, V>(pa0 + 2 * (int64_t)r * S, ar[g], ai[g]);
                        load_cvec<T, V>(psi + 2 * ((int64_t)(baseB + (uint64_t)(r ^ xl)) * S + t0), br[g], bi[g]);
                    }
                }
#pragma unroll
                for (int g = 0; g < RG; ++g)
                {
                    const int r = r0 + g;
                    if (r < RB)
                    {
                        T qr[V], qi[V];
#pragma unroll
                        for (int v = 0; v < V; ++v)
                        {
                            qr[v] = fma(ar[g][v], br[g][v], ai[g][v] * bi[g][v]);
                            qi[v] = fma(ar[g][v], bi[g][v], -(ai[g][v] * br[g][v]));
                        }
#pragma unroll
                        for (int k = 0; k < GE; ++k)
#pragma unroll
                            for (int v = 0; v < V; ++v)
                                bs[k][v] += flip_sign(qr[v], mk[k], r);
#pragma unroll
                        for (int k = 0; k < GO; ++k)
#pragma unroll
                            for (int v = 0; v < V; ++v)
                                bs[GE + k][v] += flip_sign(qi[v], mk[GE + k], r);
                    }
                }
            }
#pragma unroll
            for (int k = 0; k < G; ++k)
#pragma unroll
                for (int v = 0; v < V; ++v)
                {
                    if constexpr (sizeof(T) == 8)
                    {
                        acc[k][v] += bs[k][v];
                    }
                    else
                    {
                        // Kahan (compensated) summation of the block sums
                        const T y = bs[k][v] - cmp[k][v];
                        const T s = acc[k][v] + y;
                        cmp[k][v] = (s - acc[k][v]) - y;
                        acc[k][v] = s;
                    }
                }
        }
    }

    // deterministic float64 reduction over the row lanes, then write
    const int W = TC * V;
#pragma unroll
    for (int k = 0; k < G; ++k)
    {
        const bool valid = (k < GE) ? (k < ne) : (k - GE < no);
        if (!valid) // uniform across the CTA
            continue;
#pragma unroll
        for (int v = 0; v < V; ++v)
            red[tr * W + tc * V + v] = (double)acc[k][v] - (double)cmp[k][v];
        __syncthreads();
        for (int s = TR >> 1; s > 0; s >>= 1)
        {
            if (tr < s)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    red[tr * W + tc * V + v] += red[(tr + s) * W + tc * V + v];
            __syncthreads();
        }
        if (tr == 0 && col_ok)
        {
            const int sidx = (k < GE) ? (ch.begin_even + k) : (ch.begin_odd + (k - GE));
            const int ny = (int)(recs[sidx].meta & 3u);
            const double f = ((ny & 2) ? -1.0 : 1.0) * (paired ? 2.0 : 1.0);
            const int64_t o = orig[sidx];
            double *dst = out + ((int64_t)split * P + o) * S + t0;
#pragma unroll
            for (int v = 0; v < V; ++v)
                dst[v] = f * red[tc * V + v];
        }
        __syncthreads();
    }
}

} // namespace fpg
