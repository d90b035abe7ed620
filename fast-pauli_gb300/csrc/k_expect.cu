// k_expect.cu -- per-string expectation values <psi_t|P_j|psi_t>.
//
// Replaces the per-string stage of the reference's expectation paths
// (PauliString::expectation_value, fast_pauli/cpp/include/__pauli_string.hpp:471-538,
// called per string by SummedPauliOp::expectation_value,
// __summed_pauli_op.hpp:572-577, and PauliOp::expectation_value,
// __pauli_op.hpp:519-529).  The reference rebuilds the sparse pattern of each
// string and streams the whole state once per string; here:
//
//  * strings are grouped by x mask; a CTA serves a "chunk" of up to GE strings
//    with even #Y and GO with odd #Y from one group, so each row pair
//    (i, i^x) is loaded once for all of them;
//  * q(i) = conj(psi_i) psi_{i^x}; for even #Y a string needs Re q, for odd
//    #Y Im q, because Pauli strings are Hermitian:
//        <P> = f * sum_i (-1)^popc(i&z) v(i),  v = Re q (nY even) | Im q (odd),
//        f = +1 for nY%4 in {0,1}, -1 for nY%4 in {2,3};
//    for x >= 32 the rows with bit hb(x) clear are paired with their partner
//    and each pair contributes 2 * s(i) v(i), halving the work;
//  * the sign (-1)^popc(i&z) comes from a per-string 32-bit mask of the low
//    five row bits, xor-ed with one popcount parity per 32-row block, so the
//    inner loop has no popcount;
//  * float32 path: plain float32 sums inside a 32-row block, Kahan-compensated
//    float32 across blocks, float64 across threads and CTAs.  float64 path:
//    float64 throughout.
//
// Thread layout: TC column lanes (coalesced, V complex elements each) x
// (256 / TC) row lanes; grid = (chunks, row splits, column tiles), chunks
// fastest so that concurrently running CTAs share the state's columns in L2.
#include "common.cuh"

namespace fpg
{

const ChunkClass kChunkClasses[kNumChunkClasses] = {{1, 0}, {0, 1}, {1, 1}, {2, 2}, {4, 4}, {8, 8}, {8, 0}, {0, 8}};

int chunk_class_for(int n_even, int n_odd)
{
    int best = -1, best_cost = 1 << 30;
    for (int c = 0; c < kNumChunkClasses; ++c)
    {
        const ChunkClass k = kChunkClasses[c];
        if (k.ge >= n_even && k.go >= n_odd)
        {
            const int cost = k.ge + k.go;
            if (cost < best_cost)
            {
                best = c;
                best_cost = cost;
            }
        }
    }
    return best;
}

namespace
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

template <typename T, int V, int GE, int GO>
__global__ void __launch_bounds__(256)
    k_expect_chunks(const T *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                    const int32_t *__restrict__ orig, int64_t P, const Chunk *__restrict__ chunks, int TC,
                    int n_splits, double *__restrict__ out)
{
    constexpr int G = GE + GO;
    extern __shared__ double red[]; // blockDim.x * V doubles

    const Chunk ch = chunks[blockIdx.x];
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const int64_t t0 = ((int64_t)blockIdx.z * TC + tc) * V;
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
    const int64_t b0 = (int64_t)blockIdx.y * per;
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

    // accumulators: float64 path accumulates directly; float32 path keeps a
    // per-block float32 sum and a Kahan pair across blocks.
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
#pragma unroll
            for (int r = 0; r < 32; ++r)
            {
                if (r < RB)
                {
                    T ar[V], ai[V], br[V], bi[V];
                    load_cvec<T, V>(pa0 + 2 * (int64_t)r * S, ar, ai);
                    load_cvec<T, V>(psi + 2 * ((int64_t)(baseB + (uint64_t)(r ^ xl)) * S + t0), br, bi);
                    T qr[V], qi[V];
#pragma unroll
                    for (int v = 0; v < V; ++v)
                    {
                        qr[v] = fma(ar[v], br[v], ai[v] * bi[v]);
                        qi[v] = fma(ar[v], bi[v], -(ai[v] * br[v]));
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
            double *dst = out + ((int64_t)blockIdx.y * P + o) * S + t0;
#pragma unroll
            for (int v = 0; v < V; ++v)
                dst[v] = f * red[tc * V + v];
        }
        __syncthreads();
    }
}

template <typename T, int V>
cudaError_t launch_v(const T *psi, int64_t S, int n, const DevOp &op, const Chunk *d_chunks, int n_chunks, int cls,
                     const ExpectPlan &plan, double *out, cudaStream_t st)
{
    dim3 grid((unsigned)n_chunks, (unsigned)plan.n_splits, (unsigned)plan.n_ctiles);
    dim3 block(256);
    const size_t smem = 256 * V * sizeof(double);
#define FPG_CASE(ID, GE, GO)                                                                                           \
    case ID:                                                                                                           \
        k_expect_chunks<T, V, GE, GO><<<grid, block, smem, st>>>(psi, S, n, op.recs, op.orig, op.P, d_chunks,        \
                                                                 plan.TC, plan.n_splits, out);                       \
        break;
    switch (cls)
    {
        FPG_CASE(0, 1, 0)
        FPG_CASE(1, 0, 1)
        FPG_CASE(2, 1, 1)
        FPG_CASE(3, 2, 2)
        FPG_CASE(4, 4, 4)
        FPG_CASE(5, 8, 8)
        FPG_CASE(6, 8, 0)
        FPG_CASE(7, 0, 8)
    default:
        return cudaErrorInvalidValue;
    }
#undef FPG_CASE
    return launched();
}

__global__ void k_reduce_splits(const double *__restrict__ partial, int n_splits, int64_t count,
                                double *__restrict__ ev)
{
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    {
        double s = 0.0;
        for (int p = 0; p < n_splits; ++p)
            s += partial[(int64_t)p * count + e];
        ev[e] = s;
    }
}

} // namespace

cudaError_t launch_expect_chunks(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const Chunk *d_chunks,
                                 int n_chunks, int cls, const ExpectPlan &plan, double *out, cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    if (!fp32)
        return launch_v<double, 1>((const double *)psi, S, n, op, d_chunks, n_chunks, cls, plan, out, st);
    if (plan.V == 2)
        return launch_v<float, 2>((const float *)psi, S, n, op, d_chunks, n_chunks, cls, plan, out, st);
    return launch_v<float, 1>((const float *)psi, S, n, op, d_chunks, n_chunks, cls, plan, out, st);
}

cudaError_t launch_reduce_splits(const double *partial, int n_splits, int64_t count, double *ev, cudaStream_t st)
{
    if (count <= 0)
        return cudaSuccess;
    int64_t blocks = (count + 255) / 256;
    if (blocks > 152 * 16)
        blocks = 152 * 16;
    k_reduce_splits<<<(unsigned)blocks, 256, 0, st>>>(partial, n_splits, count, ev);
    return launched();
}

} // namespace fpg
