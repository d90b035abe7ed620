// k_expect_wht.cu -- per-string expectation values for large x-groups via a
// 16-point Walsh-Hadamard transform per row block.
//
// Same quantity as k_expect.cu (the per-string stage of
// SummedPauliOp::expectation_value, fast_pauli/cpp/include/__summed_pauli_op.hpp:572-577):
//     <P_j> = f_j * sum_i (-1)^popc(i & z_j) v(i),   v = Re or Im of conj(psi_i) psi_{i^x}.
// Split i = 16*beta + r.  Then
//     sum_i (-1)^popc(i & z) v(i) = sum_beta (-1)^popc(16 beta & z) * W_beta[z & 15],
//     W_beta[u] = sum_r (-1)^popc(r & u) v(16 beta + r)   (a 16-point WHT).
// One WHT (4 butterfly stages, 64 adds) per block serves every string of the
// group: each string then costs one shared-memory read and one add per
// 16 rows, instead of one add per row.  For a group of G strings the cost per
// row drops from ~4 + G to ~4 + 4 + G/16 operations (q, transform, lookups),
// which is what makes large groups (e.g. the 105 Z-type strings of a
// weight <= 2 set, or the 28 strings sharing one X/Y position) cheap on
// GB300's narrow float64 pipe.
//
// CTA: 128 threads = TC column lanes x TR row lanes.  A round: every row lane
// transforms one 16-row block (both parts, Re and Im, when the chunk has
// strings of both #Y parities) into shared memory; after a barrier each
// thread sums, for its own strings (string k belongs to row lane k % TR), the
// TR blocks of the round with the block-parity sign.  Each (string, column)
// accumulator lives in exactly one thread: no cross-thread reduction.
// float32 path: one Kahan-compensated add per string per round.
#include "common.cuh"

namespace fpg
{
namespace
{

template <typename T> struct C2t;
template <> struct C2t<double>
{
    using type = double2;
};
template <> struct C2t<float>
{
    using type = float2;
};

template <typename T> __device__ __forceinline__ void wht16(T (&v)[16])
{
#pragma unroll
    for (int s = 1; s < 16; s <<= 1)
#pragma unroll
        for (int r = 0; r < 16; ++r)
            if (!(r & s))
            {
                const T a = v[r], b = v[r | s];
                v[r] = a + b;
                v[r | s] = a - b;
            }
}

template <typename T, int SLOTS>
__global__ void __launch_bounds__(128)
    k_expect_wht(const T *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                 const int32_t *__restrict__ orig, int64_t P, const WhtChunk *__restrict__ chunks, int TC,
                 int n_splits, double *__restrict__ out)
{
    using CT = typename C2t<T>::type;
    extern __shared__ unsigned char smem_raw[];
    const int TR = blockDim.x / TC;
    T *wsm = reinterpret_cast<T *>(smem_raw);                  // [2][TR][16][TC]
    uint64_t *s_base = reinterpret_cast<uint64_t *>(wsm + 2 * TR * 16 * TC); // [TR], ~0 = no block
    uint64_t *s_z = s_base + TR;                                             // [count] z masks of the chunk

    const WhtChunk ch = chunks[blockIdx.x];
    const int tid = threadIdx.x;
    const int tc = tid % TC;
    const int tr = tid / TC;
    const int64_t t0 = (int64_t)blockIdx.z * TC + tc;
    const bool col_ok = t0 < S;
    const uint64_t D = 1ull << n;
    const uint64_t xh = ch.x & ~15ull;
    const uint32_t xl = (uint32_t)ch.x & 15u;
    const bool paired = xh != 0;
    const int64_t NB = n >= 4 ? (int64_t)(D >> 4) : 1;
    const int RB = n >= 4 ? 16 : (int)D;
    const int64_t nblk = paired ? NB / 2 : NB;
    const int hb = paired ? (63 - __clzll((long long)(xh >> 4))) : 0;
    const int64_t per = (nblk + n_splits - 1) / n_splits;
    const int64_t b0 = (int64_t)blockIdx.y * per;
    const int64_t b1 = min(nblk, b0 + per);
    const int G = ch.count;
    const bool need_re = ch.n_even > 0, need_im = ch.n_even < G;

    // chunk strings' z masks in shared memory; this thread owns k = tr + j * TR
    for (int k = tid; k < G; k += blockDim.x)
        s_z[k] = recs[ch.begin + k].z;
    T acc[SLOTS];
    T cmp[sizeof(T) == 4 ? SLOTS : 1]; // Kahan compensation (float32 only)
#pragma unroll
    for (int j = 0; j < SLOTS; ++j)
        acc[j] = T(0);
#pragma unroll
    for (int j = 0; j < (int)(sizeof(cmp) / sizeof(T)); ++j)
        cmp[j] = T(0);
    __syncthreads();

    for (int64_t mr = b0; mr < b1; mr += TR)
    {
        const int64_t m = mr + tr;
        T vre[16], vim[16];
#pragma unroll
        for (int r = 0; r < 16; ++r)
        {
            vre[r] = T(0);
            vim[r] = T(0);
        }
        uint64_t base = ~0ull;
        if (m < b1)
        {
            const uint64_t um = (uint64_t)m;
            const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
            base = beta << 4;
            if (col_ok)
            {
                const uint64_t baseB = base ^ xh;
                const CT *ps = reinterpret_cast<const CT *>(psi);
#pragma unroll
                for (int r = 0; r < 16; ++r)
                    if (r < RB)
                    {
                        const CT a = __ldg(ps + (int64_t)(base + r) * S + t0);
                        const CT b = __ldg(ps + (int64_t)(baseB + (uint64_t)(r ^ xl)) * S + t0);
                        if (need_re)
                            vre[r] = fma(a.x, b.x, a.y * b.y);
                        if (need_im)
                            vim[r] = fma(a.x, b.y, -(a.y * b.x));
                    }
            }
        }
        if (need_re)
            wht16(vre);
        if (need_im)
            wht16(vim);
        T *w0 = wsm + (size_t)(tr * 16) * TC + tc;             // part 0 (Re)
        T *w1 = wsm + (size_t)((TR + tr) * 16) * TC + tc;      // part 1 (Im)
#pragma unroll
        for (int u = 0; u < 16; ++u)
        {
            if (need_re)
                w0[u * TC] = vre[u];
            if (need_im)
                w1[u * TC] = vim[u];
        }
        if (tc == 0)
            s_base[tr] = base;
        __syncthreads();
        const int nb = (b1 - mr < (int64_t)TR) ? (int)(b1 - mr) : TR;
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
        {
            const int k = tr + j * TR;
            if (k >= G)
                break;
            const uint64_t z = s_z[k];
            const int part = k >= ch.n_even ? 1 : 0; // odd #Y strings read the Im transform
            const T *wp = wsm + (size_t)((part * TR * 16) + (int)(z & 15u)) * TC + tc;
            T sum = T(0);
            for (int rr = 0; rr < nb; ++rr)
            {
                const T w = wp[(size_t)rr * 16 * TC];
                sum += (__popcll(s_base[rr] & z) & 1) ? -w : w;
            }
            if constexpr (sizeof(T) == 8)
            {
                acc[j] += sum;
            }
            else
            {
                const T y = sum - cmp[j];
                const T s = acc[j] + y;
                cmp[j] = (s - acc[j]) - y;
                acc[j] = s;
            }
        }
        __syncthreads();
    }

    if (!col_ok)
        return;
#pragma unroll
    for (int j = 0; j < SLOTS; ++j)
    {
        const int k = tr + j * TR;
        if (k >= G)
            break;
        const int sidx = ch.begin + k;
        const int ny = (int)(recs[sidx].meta & 3u);
        const double f = ((ny & 2) ? -1.0 : 1.0) * (paired ? 2.0 : 1.0);
        double v = (double)acc[j];
        if constexpr (sizeof(T) == 4)
            v -= (double)cmp[j];
        out[((int64_t)blockIdx.y * P + orig[sidx]) * S + t0] = f * v;
    }
}

} // namespace

cudaError_t launch_expect_wht(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const WhtChunk *d_chunks,
                              int n_chunks, int max_count, int TC, int n_ctiles, int n_splits, double *out,
                              cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    const int threads = 128;
    const int TR = threads / TC;
    const int slots_needed = (max_count + TR - 1) / TR;
    const size_t smem = (size_t)2 * TR * 16 * TC * (fp32 ? 4 : 8) + (size_t)TR * 8 + (size_t)max_count * 8;
    dim3 grid((unsigned)n_chunks, (unsigned)n_splits, (unsigned)n_ctiles);
#define FPG_WHT(SL)                                                                                                    \
    if (fp32)                                                                                                          \
        k_expect_wht<float, SL><<<grid, threads, smem, st>>>((const float *)psi, S, n, op.recs, op.orig, op.P,        \
                                                             d_chunks, TC, n_splits, out);                            \
    else                                                                                                               \
        k_expect_wht<double, SL><<<grid, threads, smem, st>>>((const double *)psi, S, n, op.recs, op.orig, op.P,      \
                                                              d_chunks, TC, n_splits, out);
    if (slots_needed <= 8)
    {
        FPG_WHT(8)
    }
    else if (slots_needed <= 32)
    {
        FPG_WHT(32)
    }
    else
        return cudaErrorInvalidValue;
#undef FPG_WHT
    return launched();
}

} // namespace fpg
