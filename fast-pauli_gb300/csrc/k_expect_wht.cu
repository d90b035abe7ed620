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
// weight <= 2 set) cheap.
//
// CTA: kWhtThreads = TC column lanes x TR row lanes.  A round: every row lane
// transforms one 16-row block (both parts, Re and Im, when the chunk has
// strings of both #Y parities) into shared memory; after a barrier each
// thread sums, for its own strings (string k belongs to row lane k % TR), the
// TR blocks of the round with the block-parity sign.  Each (string, column)
// accumulator lives in exactly one thread: no cross-thread reduction.
//
// Arithmetic (the policy W): complex64 states in float32 with one
// Kahan-compensated add per string per round; complex128 states in
// double-float (df64.cuh) on the float32 pipes, the state split once per call
// (k_df_split), followed by the float64 form, which recomputes only when the
// call's range flag was raised.
#include <type_traits>

#include "common.cuh"
#include "df64.cuh"

namespace fpg
{
namespace
{

struct DFv
{
    float h, l;
};

// complex64 states
struct W32
{
    using in_t = float2;
    using val = float;
    using cell = float; // shared-memory type of a transform value
    struct acc
    {
        float v, c;
    };
    static constexpr bool kRecompute = false;
    // the two-level transform also with 16 row lanes (its 16-point second
    // level spills the df64 and float64 forms)
    static constexpr bool kTwoLevel16 = true;
    static __device__ __forceinline__ val zero()
    {
        return 0.f;
    }
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi)
    {
        qv(__ldg(psi + ea), __ldg(psi + eb), re, im, vr, vi);
    }
    static __device__ __forceinline__ void qv(in_t a, in_t b, bool re, bool im, val &vr, val &vi)
    {
        if (re)
            vr = fmaf(a.x, b.x, a.y * b.y);
        if (im)
            vi = fmaf(a.x, b.y, -(a.y * b.x));
    }
    static __device__ __forceinline__ void butterfly(val &a, val &b)
    {
        const val s = a + b, d = a - b;
        a = s;
        b = d;
    }
    static __device__ __forceinline__ cell to_cell(val v)
    {
        return v;
    }
    static __device__ __forceinline__ val from_cell(cell c)
    {
        return c;
    }
    static __device__ __forceinline__ void add_cell(val &s, cell c, bool neg)
    {
        s += neg ? -c : c;
    }
    static __device__ __forceinline__ acc acc_zero()
    {
        return acc{0.f, 0.f};
    }
    static __device__ __forceinline__ void acc_add(acc &a, val x)
    {
        const float y = x - a.c;
        const float s = a.v + y;
        a.c = (s - a.v) - y;
        a.v = s;
    }
    static __device__ __forceinline__ double to_double(const acc &a)
    {
        return (double)a.v - (double)a.c;
    }
};

// complex128 states, float64 arithmetic (the recomputation)
struct W64
{
    using in_t = double2;
    using val = double;
    using cell = double;
    using acc = double;
    static constexpr bool kRecompute = true;
    // the two-level transform also with 16 row lanes (its 16-point second
    // level spills the df64 and float64 forms)
    static constexpr bool kTwoLevel16 = false;
    static __device__ __forceinline__ val zero()
    {
        return 0.0;
    }
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi)
    {
        qv(__ldg(psi + ea), __ldg(psi + eb), re, im, vr, vi);
    }
    static __device__ __forceinline__ void qv(in_t a, in_t b, bool re, bool im, val &vr, val &vi)
    {
        if (re)
            vr = fma(a.x, b.x, a.y * b.y);
        if (im)
            vi = fma(a.x, b.y, -(a.y * b.x));
    }
    static __device__ __forceinline__ void butterfly(val &a, val &b)
    {
        const val s = a + b, d = a - b;
        a = s;
        b = d;
    }
    static __device__ __forceinline__ cell to_cell(val v)
    {
        return v;
    }
    static __device__ __forceinline__ val from_cell(cell c)
    {
        return c;
    }
    static __device__ __forceinline__ void add_cell(val &s, cell c, bool neg)
    {
        s += neg ? -c : c;
    }
    static __device__ __forceinline__ acc acc_zero()
    {
        return 0.0;
    }
    static __device__ __forceinline__ void acc_add(acc &a, val x)
    {
        a += x;
    }
    static __device__ __forceinline__ double to_double(const acc &a)
    {
        return a;
    }
};

// complex128 states split into df64 (float4 per element): df64 arithmetic
struct WDF
{
    using in_t = float4;
    using val = DFv;
    using cell = float2;
    using acc = DFv;
    static constexpr bool kRecompute = false;
    // the two-level transform also with 16 row lanes (its 16-point second
    // level spills the df64 and float64 forms)
    static constexpr bool kTwoLevel16 = false;
    static __device__ __forceinline__ val zero()
    {
        return DFv{0.f, 0.f};
    }
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi)
    {
        qv(__ldg(psi + ea), __ldg(psi + eb), re, im, vr, vi);
    }
    static __device__ __forceinline__ void qv(in_t a, in_t b, bool re, bool im, val &vr, val &vi)
    {
        if (re)
        {
            df_mul(a.x, a.y, b.x, b.y, vr.h, vr.l);
            df_fma(a.z, a.w, b.z, b.w, vr.h, vr.l);
        }
        if (im)
        {
            df_mul(a.x, a.y, b.z, b.w, vi.h, vi.l);
            df_fma(-a.z, -a.w, b.x, b.y, vi.h, vi.l);
        }
    }
    // four levels of butterflies without renormalising (each value's low
    // part absorbs four exact errors), renormalised once as a cell
    static __device__ __forceinline__ void butterfly(val &a, val &b)
    {
        DFv s = a, d = a;
        df_add_lazy(s.h, s.l, b.h, b.l);
        df_add_lazy(d.h, d.l, -b.h, -b.l);
        a = s;
        b = d;
    }
    static __device__ __forceinline__ cell to_cell(val v)
    {
        df_norm(v.h, v.l);
        return make_float2(v.h, v.l);
    }
    static __device__ __forceinline__ val from_cell(cell c)
    {
        return DFv{c.x, c.y};
    }
    static __device__ __forceinline__ void add_cell(val &s, cell c, bool neg)
    {
        df_add(s.h, s.l, neg ? -c.x : c.x, neg ? -c.y : c.y);
    }
    static __device__ __forceinline__ acc acc_zero()
    {
        return DFv{0.f, 0.f};
    }
    static __device__ __forceinline__ void acc_add(acc &a, val x)
    {
        df_add(a.h, a.l, x.h, x.l);
    }
    static __device__ __forceinline__ double to_double(const acc &a)
    {
        return df_to_double(a.h, a.l);
    }
};

template <typename W> __device__ __forceinline__ void wht16(typename W::val (&v)[16])
{
#pragma unroll
    for (int s = 1; s < 16; s <<= 1)
#pragma unroll
        for (int r = 0; r < 16; ++r)
            if (!(r & s))
                W::butterfly(v[r], v[r | s]);
}

// q of the block's 16 rows into vr / vi (one array when !BOTH: each row's
// single part), the loads of four row pairs issued before any of them is
// used; for the diagonal group (each row paired with itself) one load per row,
// eight rows at a time for 8-byte elements and four for 16-byte ones (eight
// of those spill).  OFF32 (n >= 4, 16 S < 2^31): row r of a block is loaded
// at the block's first element plus r S in 32 bits, one wide multiply-add
// per load, instead of 64-bit index arithmetic per row.
template <typename W, bool BOTH, bool OFF32>
__device__ __forceinline__ void rows_q(const typename W::in_t *__restrict__ psi, int64_t S, int64_t t0, uint64_t base,
                                       uint64_t baseB, uint32_t xl, int RB, bool need_re, bool need_im,
                                       typename W::val (&vr)[16], typename W::val (&vi)[16])
{
    if constexpr (OFF32)
    {
        const int S32 = (int)S;
        const typename W::in_t *qa = psi + ((int64_t)base * S + t0);
        if (xl == 0u && baseB == base)
        {
            constexpr int RGD = sizeof(typename W::in_t) <= 8 ? 8 : 4;
#pragma unroll
            for (int r0 = 0; r0 < 16; r0 += RGD)
            {
                typename W::in_t a[RGD];
#pragma unroll
                for (int u = 0; u < RGD; ++u)
                    a[u] = __ldg(qa + (r0 + u) * S32);
#pragma unroll
                for (int u = 0; u < RGD; ++u)
                    W::qv(a[u], a[u], need_re, need_im, vr[r0 + u], vi[r0 + u]);
            }
            return;
        }
        const typename W::in_t *qb = psi + ((int64_t)baseB * S + t0);
#pragma unroll
        for (int r0 = 0; r0 < 16; r0 += 4)
        {
            typename W::in_t a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                a[u] = __ldg(qa + (r0 + u) * S32);
                b[u] = __ldg(qb + (int)((uint32_t)(r0 + u) ^ xl) * S32);
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                W::qv(a[u], b[u], need_re, need_im, vr[r0 + u], vi[r0 + u]);
        }
        return;
    }
    if (xl == 0u && baseB == base)
    {
        constexpr int RGD = sizeof(typename W::in_t) <= 8 ? 8 : 4;
#pragma unroll
        for (int r0 = 0; r0 < 16; r0 += RGD)
        {
            typename W::in_t a[RGD];
#pragma unroll
            for (int u = 0; u < RGD; ++u)
                if (r0 + u < RB)
                    a[u] = __ldg(psi + (int64_t)(base + r0 + u) * S + t0);
#pragma unroll
            for (int u = 0; u < RGD; ++u)
                if (r0 + u < RB)
                    W::qv(a[u], a[u], need_re, need_im, vr[r0 + u], vi[r0 + u]);
        }
        return;
    }
#pragma unroll
    for (int r0 = 0; r0 < 16; r0 += 4)
    {
        typename W::in_t a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (r0 + u < RB)
            {
                a[u] = __ldg(psi + (int64_t)(base + r0 + u) * S + t0);
                b[u] = __ldg(psi + (int64_t)(baseB + (uint64_t)((r0 + u) ^ xl)) * S + t0);
            }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (r0 + u < RB)
                W::qv(a[u], b[u], need_re, need_im, vr[r0 + u], vi[r0 + u]);
    }
}

// Second level: in place over the round's TR2 blocks, for every (part,
// coefficient u, column lane): W2[v] = sum_rr (-1)^popc(rr & v) W[rr].
template <typename W, int TR2>
__device__ __forceinline__ void wht_rounds(typename W::cell *wsm, int TR, int TC, int first_part, int parts)
{
    using val = typename W::val;
    for (int idx = threadIdx.x; idx < parts * 16 * TC; idx += blockDim.x)
    {
        const int pi = idx / (16 * TC), rem = idx - pi * 16 * TC;
        const int part = first_part + pi;
        typename W::cell *c0 = wsm + (size_t)part * TR * 16 * TC + rem; // + rr * 16 * TC
        val v[TR2];
#pragma unroll
        for (int rr = 0; rr < TR2; ++rr)
            v[rr] = W::from_cell(c0[(size_t)rr * 16 * TC]);
#pragma unroll
        for (int st = 1; st < TR2; st <<= 1)
#pragma unroll
            for (int rr = 0; rr < TR2; ++rr)
                if (!(rr & st))
                    W::butterfly(v[rr], v[rr | st]);
#pragma unroll
        for (int rr = 0; rr < TR2; ++rr)
            c0[(size_t)rr * 16 * TC] = W::to_cell(v[rr]);
    }
}

// only_if: when not null, the float64 recomputation returns at once unless
// *only_if is set.
// BOTH: some chunk of the launch has strings of both #Y parities (two
// transforms per block); otherwise one.
template <typename W, int SLOTS, bool BOTH, bool OFF32>
__global__ void __launch_bounds__(kWhtThreads, BOTH ? 1 : 2)
    k_expect_wht(const typename W::in_t *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                 const int32_t *__restrict__ orig, int64_t P, const WhtChunk *__restrict__ chunks, int TC,
                 int n_splits, double *__restrict__ out, const int *__restrict__ only_if)
{
    using val = typename W::val;
    using cell = typename W::cell;
    using acc = typename W::acc;
    if (W::kRecompute && only_if && *only_if == 0)
        return;
    extern __shared__ unsigned char smem_raw[];
    const int TR = blockDim.x / TC;
    cell *wsm = reinterpret_cast<cell *>(smem_raw);                                // [2][TR][16][TC]
    uint64_t *s_base = reinterpret_cast<uint64_t *>(smem_raw + (size_t)2 * TR * 16 * TC * 8); // [TR], ~0 = no block
    uint64_t *s_z = s_base + TR;                                                   // [count] z masks of the chunk

    const WhtChunk ch = chunks[blockIdx.x];
    // [count] per string: bit rr = parity(base of block rr & z), the block's
    // sign, computed once per CTA instead of once per column lane
    uint32_t *s_sign = reinterpret_cast<uint32_t *>(s_z + ch.count);
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
    // rows per split in whole rounds, so that a round's blocks are TR
    // consecutive, TR-aligned block indices
    const int64_t per = ((nblk + n_splits - 1) / n_splits + TR - 1) / TR * TR;
    const int64_t b0 = (int64_t)blockIdx.y * per;
    const int64_t b1 = min(nblk, b0 + per);
    const int G = ch.count;
    const bool need_re = ch.n_even > 0, need_im = ch.n_even < G;
    // two levels: x below the block (x < 16) and TR = 8 row lanes (or 16, in
    // the float32 form) --
    // the round's TR blocks differ only in block-index bits below log2 TR
    // (row bits 4..), so a string's sign over them factors as
    // (-1)^popc(base_0 & z) times the TR-point Walsh-Hadamard kernel at
    // (z >> 4) & (TR - 1): one more TR-point transform per (coefficient,
    // column) and a round costs each string one read instead of TR signed
    // adds (16 row lanes: the float32 form at n = 18, whose column tile of 16
    // lanes fits the L2 budget)
    const bool two_level = !paired && (TR == 8 || (W::kTwoLevel16 && TR == 16));

    // chunk strings' z masks in shared memory; this thread owns k = tr + j * TR
    for (int k = tid; k < G; k += blockDim.x)
        s_z[k] = recs[ch.begin + k].z;
    acc sums[SLOTS];
#pragma unroll
    for (int j = 0; j < SLOTS; ++j)
        sums[j] = W::acc_zero();
    __syncthreads();

    for (int64_t mr = b0; mr < b1; mr += TR)
    {
        const int64_t m = mr + tr;
        uint64_t base = ~0ull;
        const bool have = m < b1;
        if (have)
        {
            const uint64_t um = (uint64_t)m;
            const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
            base = beta << 4;
        }
        const uint64_t baseB = base ^ xh;
        cell *w0 = wsm + (size_t)(tr * 16) * TC + tc;        // part 0 (Re)
        cell *w1 = wsm + (size_t)((TR + tr) * 16) * TC + tc; // part 1 (Im)
        if constexpr (BOTH)
        {
            val vre[16], vim[16];
#pragma unroll
            for (int r = 0; r < 16; ++r)
            {
                vre[r] = W::zero();
                vim[r] = W::zero();
            }
            if (have && col_ok)
                rows_q<W, true, OFF32>(psi, S, t0, base, baseB, xl, RB, need_re, need_im, vre, vim);
            if (need_re)
                wht16<W>(vre);
            if (need_im)
                wht16<W>(vim);
#pragma unroll
            for (int u = 0; u < 16; ++u)
            {
                if (need_re)
                    w0[u * TC] = W::to_cell(vre[u]);
                if (need_im)
                    w1[u * TC] = W::to_cell(vim[u]);
            }
        }
        else
        {
            // every string of the chunk reads the same part: one transform
            val v[16];
#pragma unroll
            for (int r = 0; r < 16; ++r)
                v[r] = W::zero();
            if (have && col_ok)
                rows_q<W, false, OFF32>(psi, S, t0, base, baseB, xl, RB, need_re, need_im, v, v);
            wht16<W>(v);
            cell *w = need_re ? w0 : w1;
#pragma unroll
            for (int u = 0; u < 16; ++u)
                w[u * TC] = W::to_cell(v[u]);
        }
        if (tc == 0)
            s_base[tr] = base;
        __syncthreads();
        if (two_level)
        {
            // the parts written above: both, or the one the chunk's strings read
            if constexpr (W::kTwoLevel16)
            {
                if (TR == 16)
                    wht_rounds<W, 16>(wsm, TR, TC, BOTH ? 0 : (need_re ? 0 : 1), BOTH ? 2 : 1);
                else
                    wht_rounds<W, 8>(wsm, TR, TC, BOTH ? 0 : (need_re ? 0 : 1), BOTH ? 2 : 1);
            }
            else
                wht_rounds<W, 8>(wsm, TR, TC, BOTH ? 0 : (need_re ? 0 : 1), BOTH ? 2 : 1);
            __syncthreads();
            const uint64_t base0 = s_base[0];
#pragma unroll
            for (int j = 0; j < SLOTS; ++j)
            {
                const int k = tr + j * TR;
                if (k >= G)
                    break;
                const uint64_t z = s_z[k];
                // with one transform (!BOTH) its cells sit in the part the
                // chunk's strings read
                const int part = BOTH ? (k >= ch.n_even ? 1 : 0) : (need_re ? 0 : 1);
                const cell c =
                    wsm[(size_t)(((part * TR + (int)((z >> 4) & (uint64_t)(TR - 1))) * 16) + (int)(z & 15u)) * TC + tc];
                val sum = W::zero();
                W::add_cell(sum, c, (__popcll(base0 & z) & 1) != 0);
                W::acc_add(sums[j], sum);
            }
            __syncthreads();
            continue;
        }
        const int nb = (b1 - mr < (int64_t)TR) ? (int)(b1 - mr) : TR;
        const bool masks = TR <= 32; // one bit per block of the round
        for (int k = tid; masks && k < G; k += blockDim.x)
        {
            const uint64_t z = s_z[k];
            uint32_t sg = 0;
            for (int rr = 0; rr < nb; ++rr)
                sg |= (uint32_t)(__popcll(s_base[rr] & z) & 1) << rr;
            s_sign[k] = sg;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < SLOTS; ++j)
        {
            const int k = tr + j * TR;
            if (k >= G)
                break;
            const uint64_t z = s_z[k];
            const uint32_t sg = masks ? s_sign[k] : 0u;
            const int part = k >= ch.n_even ? 1 : 0; // odd #Y strings read the Im transform
            const cell *wp = wsm + (size_t)((part * TR * 16) + (int)(z & 15u)) * TC + tc;
            val sum = W::zero();
            for (int rr = 0; rr < nb; ++rr)
                W::add_cell(sum, wp[(size_t)rr * 16 * TC],
                            masks ? ((sg >> rr) & 1u) != 0 : (__popcll(s_base[rr] & z) & 1) != 0);
            W::acc_add(sums[j], sum);
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
        out[((int64_t)blockIdx.y * P + orig[sidx]) * S + t0] = f * W::to_double(sums[j]);
    }
}

template <typename W, int SL, bool BOTH, bool OFF32>
cudaError_t launch_w_off(const void *psi, int64_t S, int n, const DevOp &op, const WhtChunk *d_chunks, int n_chunks,
                         int TC, int n_ctiles, int n_splits, double *out, const int *only_if, size_t smem,
                         cudaStream_t st)
{
    dim3 grid((unsigned)n_chunks, (unsigned)n_splits, (unsigned)n_ctiles);
    cudaError_t e = cudaFuncSetAttribute(k_expect_wht<W, SL, BOTH, OFF32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess)
        return e;
    k_expect_wht<W, SL, BOTH, OFF32><<<grid, kWhtThreads, smem, st>>>(
        (const typename W::in_t *)psi, S, n, op.recs, op.orig, op.P, d_chunks, TC, n_splits, out, only_if);
    return launched();
}

// 32-bit row offsets for the float32 form (W32) of whole 16-row blocks
template <typename W, int SL, bool BOTH>
cudaError_t launch_w(const void *psi, int64_t S, int n, const DevOp &op, const WhtChunk *d_chunks, int n_chunks,
                     int TC, int n_ctiles, int n_splits, double *out, const int *only_if, size_t smem, cudaStream_t st)
{
    if constexpr (std::is_same_v<W, W32>)
        if (n >= 4 && 16 * S < ((int64_t)1 << 31))
            return launch_w_off<W, SL, BOTH, true>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out,
                                                   only_if, smem, st);
    return launch_w_off<W, SL, BOTH, false>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, only_if,
                                            smem, st);
}

template <int SL, bool BOTH>
cudaError_t launch_sl(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const WhtChunk *d_chunks,
                      int n_chunks, int TC, int n_ctiles, int n_splits, double *out, int *range_flag,
                      const void *psi_df, size_t smem, cudaStream_t st)
{
    if (fp32)
        return launch_w<W32, SL, BOTH>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, nullptr, smem,
                                       st);
    if (psi_df)
    {
        if (cudaError_t e = launch_w<WDF, SL, BOTH>(psi_df, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out,
                                                    nullptr, smem, st))
            return e;
        return launch_w<W64, SL, BOTH>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag,
                                       smem, st);
    }
    // no df64 copy of the state: float64 throughout
    return launch_w<W64, SL, BOTH>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, nullptr, smem, st);
}

} // namespace

cudaError_t launch_expect_wht(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const WhtChunk *d_chunks,
                              int n_chunks, int max_count, bool both_parts, int TC, int n_ctiles, int n_splits,
                              double *out, int *range_flag, const void *psi_df, cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    const int threads = kWhtThreads;
    const int TR = threads / TC;
    const int slots_needed = (max_count + TR - 1) / TR;
    const size_t smem = (size_t)2 * TR * 16 * TC * 8 + (size_t)TR * 8 + (size_t)max_count * 12;
#define FPG_WHT(SL, BOTH)                                                                                              \
    return launch_sl<SL, BOTH>(fp32, psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag,     \
                               psi_df, smem, st)
    if (slots_needed <= 8)
    {
        if (both_parts)
            FPG_WHT(8, true);
        FPG_WHT(8, false);
    }
    if (slots_needed <= 16)
    {
        if (both_parts)
            FPG_WHT(16, true);
        FPG_WHT(16, false);
    }
#undef FPG_WHT
    return cudaErrorInvalidValue; // TR >= 8 and <= kWhtMaxStrings strings: at most 16 slots
}

} // namespace fpg
