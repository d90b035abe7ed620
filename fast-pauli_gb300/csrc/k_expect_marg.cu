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
// set in the block's base.
//
// Rows: as k_expect_pair.cu -- blocks paired for x >= 32, rows paired inside
// a block for 0 < x < 32 (16 rows visited), all rows for x = 0.  Layout: TC
// column lanes x (256 / TC) row lanes, one complex element per lane; grid
// (chunks, row splits, column tiles).
//
// Arithmetic (the policy A):
//  * complex64 states: float32 sums inside a block, Kahan-compensated float32
//    across blocks, float64 across threads;
//  * complex128 states: double-float (df64.cuh) throughout the block and
//    across blocks -- the float64 result to ~2^-46 of sum |terms| at float32
//    pipe rates -- and float64 across threads.
#include <type_traits>

#include "df64.cuh"

#include "expect_body.cuh"

namespace fpg
{
namespace
{

struct DF
{
    float h, l;
};

// complex64 states: float values, Kahan accumulators
struct ArF32
{
    using in_t = float;
    static constexpr bool kRaises = false, kRecompute = false;
    using val = float;
    struct acc
    {
        float v, c;
    };
    static __device__ __forceinline__ val zero()
    {
        return 0.f;
    }
    static __device__ __forceinline__ void add(val &a, val b)
    {
        a += b;
    }
    static __device__ __forceinline__ void fix(val &)
    {
    }
    static __device__ __forceinline__ val sum(val a, val b)
    {
        return a + b;
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
    // the row-lane reduction in double-float pairs (hi, lo) on the float32 pipes
    static constexpr bool kPairReduce = true;
    static __device__ __forceinline__ float2 to_pair(const acc &a)
    {
        return make_float2(a.v, -a.c);
    }
    // a += b (both compensated: b's sum is b.v - b.c)
    static __device__ __forceinline__ void acc_merge(acc &a, const acc &b)
    {
        acc_add(a, b.v);
        acc_add(a, -b.c);
    }
    static __device__ __forceinline__ acc from2(float2 f)
    {
        return acc{f.x, f.y};
    }
    static __device__ __forceinline__ float2 to2(const acc &a)
    {
        return make_float2(a.v, a.c);
    }
    // q = conj(psi_a) psi_b at element pointers pa, pb
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi, bool &)
    {
        const float2 a = __ldg(reinterpret_cast<const float2 *>(psi) + ea);
        const float2 b = __ldg(reinterpret_cast<const float2 *>(psi) + eb);
        qraw(a, b, re, im, vr, vi);
    }
    // small elements: a block half's 32 loads are issued before any use
    static constexpr int kPrefetchRows = 16;
    static constexpr int kBatchUnroll = 4;
    // row offsets from the CTA's table: 2.56 -> 1.92 ms per n=18 launch
    static constexpr bool kRowTable = true;
    using raw_t = float2;
    static __device__ __forceinline__ raw_t ld(const in_t *psi, int64_t e)
    {
        return __ldg(reinterpret_cast<const float2 *>(psi) + e);
    }
    static __device__ __forceinline__ raw_t raw_zero()
    {
        return make_float2(0.f, 0.f);
    }
    static __device__ __forceinline__ void qraw(raw_t a, raw_t b, bool re, bool im, val &vr, val &vi)
    {
        if (re)
            vr = fmaf(a.x, b.x, a.y * b.y);
        if (im)
            vi = fmaf(a.x, b.y, -(a.y * b.x));
    }
};

// complex128 states, float64 arithmetic: the recomputation for inputs
// outside the df64 range
struct ArF64
{
    using in_t = double;
    static constexpr bool kRaises = false, kRecompute = true;
    static constexpr int kPrefetchRows = 0;
    static constexpr int kBatchUnroll = 4;
    static constexpr bool kRowTable = false;
    using raw_t = double2;
    static __device__ __forceinline__ raw_t ld(const in_t *, int64_t)
    {
        return make_double2(0.0, 0.0);
    }
    static __device__ __forceinline__ raw_t raw_zero()
    {
        return make_double2(0.0, 0.0);
    }
    using val = double;
    using acc = double;
    static __device__ __forceinline__ val zero()
    {
        return 0.0;
    }
    static __device__ __forceinline__ void add(val &a, val b)
    {
        a += b;
    }
    static __device__ __forceinline__ void fix(val &)
    {
    }
    static __device__ __forceinline__ val sum(val a, val b)
    {
        return a + b;
    }
    static __device__ __forceinline__ acc acc_zero()
    {
        return 0.0;
    }
    static __device__ __forceinline__ void acc_add(acc &a, val x)
    {
        a += x;
    }
    static __device__ __forceinline__ void acc_merge(acc &a, const acc &b)
    {
        a += b;
    }
    static __device__ __forceinline__ double to_double(const acc &a)
    {
        return a;
    }
    static constexpr bool kPairReduce = false;
    static __device__ __forceinline__ float2 to_pair(const acc &)
    {
        return make_float2(0.f, 0.f);
    }
    static __device__ __forceinline__ acc from2(float2 f)
    {
        return (double)__hiloint2double(__float_as_int(f.y), __float_as_int(f.x));
    }
    static __device__ __forceinline__ float2 to2(const acc &a)
    {
        return make_float2(__int_as_float(__double2loint(a)), __int_as_float(__double2hiint(a)));
    }
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi, bool &)
    {
        const double2 a = __ldg(reinterpret_cast<const double2 *>(psi) + ea);
        const double2 b = __ldg(reinterpret_cast<const double2 *>(psi) + eb);
        if (re)
            vr = fma(a.x, b.x, a.y * b.y);
        if (im)
            vi = fma(a.x, b.y, -(a.y * b.x));
    }
};

// complex128 states: df64 values and accumulators; raises the range flag
struct ArDF
{
    using in_t = double;
    static constexpr bool kRaises = true, kRecompute = false;
    static constexpr int kPrefetchRows = 0;
    static constexpr int kBatchUnroll = 4;
    static constexpr bool kRowTable = false;
    using raw_t = float4;
    static __device__ __forceinline__ float4 raw_zero()
    {
        return make_float4(0.f, 0.f, 0.f, 0.f);
    }
    using val = DF;
    using acc = DF;
    static __device__ __forceinline__ val zero()
    {
        return DF{0.f, 0.f};
    }
    // inside a block: sums without renormalising, fixed at each 16-row half
    static __device__ __forceinline__ void add(val &a, val b)
    {
        df_add_lazy(a.h, a.l, b.h, b.l);
    }
    static __device__ __forceinline__ val sum(val a, val b)
    {
        df_add_lazy(a.h, a.l, b.h, b.l);
        return a;
    }
    static __device__ __forceinline__ void fix(val &a)
    {
        df_norm(a.h, a.l);
    }
    static __device__ __forceinline__ acc acc_zero()
    {
        return DF{0.f, 0.f};
    }
    static __device__ __forceinline__ void acc_add(acc &a, val x)
    {
        df_add(a.h, a.l, x.h, x.l);
    }
    static __device__ __forceinline__ void acc_merge(acc &a, const acc &b)
    {
        df_add(a.h, a.l, b.h, b.l);
    }
    static __device__ __forceinline__ double to_double(const acc &a)
    {
        return df_to_double(a.h, a.l);
    }
    static constexpr bool kPairReduce = true;
    static __device__ __forceinline__ float2 to_pair(const acc &a)
    {
        return make_float2(a.h, a.l);
    }
    static __device__ __forceinline__ acc from2(float2 f)
    {
        return DF{f.x, f.y};
    }
    static __device__ __forceinline__ float2 to2(const acc &a)
    {
        return make_float2(a.h, a.l);
    }
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi, bool &bad)
    {
        const float4 a = split_complex(__ldg(reinterpret_cast<const uint4 *>(psi) + ea), bad);
        const float4 b = split_complex(__ldg(reinterpret_cast<const uint4 *>(psi) + eb), bad);
        qdf(a, b, re, im, vr, vi);
    }
    // q = conj(a) b from df64 amplitudes (re_h, re_l, im_h, im_l)
    static __device__ __forceinline__ void qdf(float4 a, float4 b, bool re, bool im, val &vr, val &vi)
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
};

// complex128 states already split into df64 (k_df_split, which also checked
// the range): the arithmetic of ArDF without the split
struct ArDFS : ArDF
{
    using in_t = float4;
    static constexpr bool kRaises = false, kRecompute = false;
    // 16-byte elements: loads issued four rows at a time ahead of use
    static constexpr int kPrefetchRows = 4;
    // the batch loop rolled and the row offsets from the CTA's table: n=14
    // weight<=2 step 2.185 -> 2.150 ms (rolled: the unrolled body missed the
    // instruction cache) -> 2.072 ms (with the table, which spilled while the
    // loop was unrolled)
    static constexpr int kBatchUnroll = 1;
    static constexpr bool kRowTable = true;
    static __device__ __forceinline__ void q(const in_t *psi, int64_t ea, int64_t eb, bool re, bool im, val &vr,
                                             val &vi, bool &)
    {
        qdf(__ldg(psi + ea), __ldg(psi + eb), re, im, vr, vi);
    }
    static __device__ __forceinline__ raw_t ld(const in_t *psi, int64_t e)
    {
        return __ldg(psi + e);
    }
    static __device__ __forceinline__ void qraw(raw_t a, raw_t b, bool re, bool im, val &vr, val &vi)
    {
        qdf(a, b, re, im, vr, vi);
    }
};

// Sums of one block: bt[part] (total) and bl[part][j] (rows whose visited-row
// bit j is set).  LB = 5: all 32 rows, visited bit j = row bit j.  LB = 4:
// the 16 rows with bit pl clear; visited bit j = row bit (j < pl ? j : j + 1).
// TAB (policies with kRowTable, n >= 5, 32 S < 2^31): the element offsets of
// the visited rows from the block's first row come from the CTA's table
// s_rows ({row, partner row} x S, 32-bit), so a row load is one wide
// multiply-add on a pointer formed once per block instead of 64-bit index
// arithmetic per row.
// BOTHP: the chunk needs both parts (need_re and need_im), known at compile
// time so that no q or tree step is conditional.
template <typename A, int LB, bool TAB, bool BOTHP>
__device__ __forceinline__ void block_marginals(const typename A::in_t *__restrict__ psi, int64_t S, int64_t t0,
                                                uint64_t base, uint64_t baseB, uint32_t xl, int pl, int RB,
                                                bool need_re_, bool need_im_, typename A::val (&bt)[2],
                                                typename A::val (&bl)[2][5], bool &bad, const int2 *s_rows)
{
    using val = typename A::val;
    const bool need_re = BOTHP || need_re_, need_im = BOTHP || need_im_;
    [[maybe_unused]] const typename A::raw_t *qa = nullptr, *qb = nullptr;
    if constexpr (TAB)
    {
        qa = reinterpret_cast<const typename A::raw_t *>(psi) + ((int64_t)base * S + t0);
        qb = reinterpret_cast<const typename A::raw_t *>(psi) + ((int64_t)baseB * S + t0);
    }
    // 16 visited rows at a time (LB = 5: two halves, bit 4 from the half)
#pragma unroll 1
    for (int h = 0; h < (1 << (LB - 4)); ++h)
    {
        val hs[2] = {A::zero(), A::zero()};
        // kPrefetchRows > 0: the loads of that many row pairs are issued
        // before any of them is used (batches of the half's 16)
        constexpr int PF = A::kPrefetchRows > 0 ? A::kPrefetchRows : 1;
        typename A::raw_t ra[PF], rb[PF];
        // the block's first rows of this column, when psi points at whole
        // elements (the df64 split copy): row loads add r * S only
        constexpr bool kElemPtr = std::is_same_v<typename A::in_t, typename A::raw_t>;
        [[maybe_unused]] const typename A::in_t *pa = psi + ((int64_t)base * S + t0);
        [[maybe_unused]] const typename A::in_t *pb = psi + ((int64_t)baseB * S + t0);
        // the half's four 4-row batches: unrolled, or (kBatchUnroll = 1) a
        // loop, for a kernel body that stays in the instruction cache
#pragma unroll(A::kBatchUnroll)
        for (int k = 0; k < 4; ++k)
        {
            if constexpr (A::kPrefetchRows > 0)
            {
                if ((4 * k) % PF == 0)
                {
#pragma unroll
                    for (int j = 0; TAB && j < PF; ++j)
                    {
                        const int2 o = s_rows[16 * h + 4 * k + j];
                        ra[j] = __ldg(qa + o.x);
                        rb[j] = __ldg(qb + o.y);
                    }
#pragma unroll
                    for (int j = 0; !TAB && j < PF; ++j)
                    {
                        const uint32_t m2 = (uint32_t)(16 * h + 4 * k + j);
                        const uint32_t r = LB == 5 ? m2 : (((m2 >> pl) << (pl + 1)) | (m2 & ((1u << pl) - 1u)));
                        ra[j] = A::raw_zero();
                        rb[j] = A::raw_zero();
                        if ((int)r < RB)
                        {
                            if constexpr (kElemPtr)
                            {
                                ra[j] = A::ld(pa, (int64_t)r * S);
                                rb[j] = A::ld(pb, (int64_t)(r ^ xl) * S);
                            }
                            else
                            {
                                ra[j] = A::ld(psi, (int64_t)(base + r) * S + t0);
                                rb[j] = A::ld(psi, (int64_t)(baseB + (r ^ xl)) * S + t0);
                            }
                        }
                    }
                }
            }
            val v[4][2];
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                v[u][0] = A::zero();
                v[u][1] = A::zero();
                if constexpr (A::kPrefetchRows > 0)
                {
                    // PF = 4: batch k's rows are ra[u] (a compile-time index
                    // whether or not the batch loop is unrolled)
                    const int ri = PF == 4 ? u : (4 * k + u) % PF;
                    A::qraw(ra[ri], rb[ri], need_re, need_im, v[u][0], v[u][1]);
                }
                else
                {
                    const uint32_t m2 = (uint32_t)(16 * h + 4 * k + u);
                    const uint32_t r = LB == 5 ? m2 : (((m2 >> pl) << (pl + 1)) | (m2 & ((1u << pl) - 1u)));
                    if ((int)r < RB)
                        A::q(psi, (int64_t)(base + r) * S + t0, (int64_t)(baseB + (r ^ xl)) * S + t0, need_re,
                             need_im, v[u][0], v[u][1], bad);
                }
            }
#pragma unroll
            for (int p = 0; p < 2; ++p)
            {
                if (p == 0 ? !need_re : !need_im)
                    continue;
                const val p0 = A::sum(v[0][p], v[1][p]);
                const val p1 = A::sum(v[2][p], v[3][p]);
                A::add(bl[p][0], v[1][p]);
                A::add(bl[p][0], v[3][p]);
                A::add(bl[p][1], p1);
                const val g = A::sum(p0, p1);
                A::add(hs[p], g);
                if (k & 1)
                    A::add(bl[p][2], g);
                if (k & 2)
                    A::add(bl[p][3], g);
            }
        }
#pragma unroll
        for (int p = 0; p < 2; ++p)
        {
            A::add(bt[p], hs[p]);
            if (h)
                A::add(bl[p][4], hs[p]);
            A::fix(bt[p]);
#pragma unroll
            for (int j = 0; j < 5; ++j)
                A::fix(bl[p][j]);
        }
    }
}

// range_flag: ArDF raises it for inputs outside the df64 range; ArF64 (the
// recomputation launched after it) returns at once unless it is set.
template <typename A, int NH, bool TAB>
__global__ void __launch_bounds__(256, 2)
    k_expect_marg(const typename A::in_t *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                  const int32_t *__restrict__ orig, int64_t P, const MargChunk *__restrict__ chunks, int TC,
                  int n_splits, double *__restrict__ out, int *__restrict__ range_flag)
{
    if (A::kRecompute && *range_flag == 0)
        return;
    bool bad = false;
    using val = typename A::val;
    using acc = typename A::acc;
    constexpr int NV = 2 * (1 + 5 + NH); // values per thread: [part][total, low 5, high NH]
    constexpr int NVB = 8;               // values reduced per pass
    extern __shared__ double smem[];
    double *red = smem;                  // [NVB][256]
    double *res = smem + NVB * 256;      // [NV][TC] totals per column lane
    float2 *smh = reinterpret_cast<float2 *>(res + NV * TC); // [2][NH][256] high-bit accumulators

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

    // row bits >= 5 used by the strings (at most NH): their marginals live in
    // shared memory, one (float, float) accumulator per thread each, added to
    // once per block
    const uint64_t hmask = ch.zmask & ~31ull;
    for (int j = 0; j < 2 * NH; ++j)
        smh[j * 256 + tid] = make_float2(0.f, 0.f);
    // visited row m2 -> element offsets of its row and partner row from the
    // block's first rows (base, baseB)
    __shared__ int2 s_rows[32];
    if constexpr (TAB)
    {
        if (tid < 32)
        {
            const uint32_t m2 = (uint32_t)tid;
            const uint32_t r = pl < 0 ? m2 : (((m2 >> pl) << (pl + 1)) | (m2 & ((1u << pl) - 1u)));
            s_rows[tid] = make_int2((int)(r & 31u) * (int)S, (int)((r ^ xl) & 31u) * (int)S);
        }
        __syncthreads();
    }

    acc tot[2], ml[2][5];
#pragma unroll
    for (int p = 0; p < 2; ++p)
    {
        tot[p] = A::acc_zero();
#pragma unroll
        for (int j = 0; j < 5; ++j)
            ml[p][j] = A::acc_zero();
    }

    auto base_of = [&](int64_t m) -> uint64_t {
        const uint64_t um = (uint64_t)m;
        const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
        return beta << 5;
    };
    // The high bits that change within this thread's next few blocks go to
    // their cells block by block (lo_mask); the others hold still over runs
    // of blocks, whose totals are summed in registers (run) and added to the
    // cells when the pattern changes -- far fewer shared-memory updates.
    uint64_t lo_mask = 0;
    if (b0 + tr < b1)
    {
        const uint64_t f = base_of(b0 + tr);
        for (int k = 1; k < 8 && b0 + tr + (int64_t)k * TR < b1; ++k)
            lo_mask |= base_of(b0 + tr + (int64_t)k * TR) ^ f;
    }
    lo_mask &= hmask;
    const uint64_t hi_mask = hmask & ~lo_mask;
    auto cell_merge = [&](int p, uint64_t bits, const acc &x) {
        for (uint64_t w = bits; w; w &= w - 1ull)
        {
            const int b = __ffsll((long long)w) - 1;
            float2 *cell = smh + (p * NH + __popcll(hmask & ((1ull << b) - 1ull))) * 256 + tid;
            acc a = A::from2(*cell);
            A::acc_merge(a, x);
            *cell = A::to2(a);
        }
    };
    acc run[2] = {A::acc_zero(), A::acc_zero()};
    uint64_t run_hi = 0;
    bool in_run = false;

    if (col_ok)
    {
        for (int64_t m = b0 + tr; m < b1; m += TR)
        {
            const uint64_t base = base_of(m);
            const uint64_t baseB = base ^ xh;
            val bt[2] = {A::zero(), A::zero()};
            val bl[2][5];
#pragma unroll
            for (int p = 0; p < 2; ++p)
#pragma unroll
                for (int j = 0; j < 5; ++j)
                    bl[p][j] = A::zero();
            if (need_re && need_im)
            {
                if (pl < 0)
                    block_marginals<A, 5, TAB, true>(psi, S, t0, base, baseB, xl, pl, RB, true, true, bt, bl, bad,
                                                     s_rows);
                else
                    block_marginals<A, 4, TAB, true>(psi, S, t0, base, baseB, xl, pl, RB, true, true, bt, bl, bad,
                                                     s_rows);
            }
            else if (pl < 0)
                block_marginals<A, 5, TAB, false>(psi, S, t0, base, baseB, xl, pl, RB, need_re, need_im, bt, bl, bad,
                                                  s_rows);
            else
                block_marginals<A, 4, TAB, false>(psi, S, t0, base, baseB, xl, pl, RB, need_re, need_im, bt, bl, bad,
                                                  s_rows);
            const uint64_t hi = base & hi_mask;
            if (in_run && hi != run_hi)
            {
#pragma unroll
                for (int p = 0; p < 2; ++p)
                {
                    cell_merge(p, run_hi, run[p]);
                    run[p] = A::acc_zero();
                }
            }
            in_run = true;
            run_hi = hi;
#pragma unroll
            for (int p = 0; p < 2; ++p)
            {
                A::acc_add(tot[p], bt[p]);
#pragma unroll
                for (int j = 0; j < 5; ++j)
                    A::acc_add(ml[p][j], bl[p][j]);
                A::acc_add(run[p], bt[p]);
                for (uint64_t w = base & lo_mask; w; w &= w - 1ull)
                {
                    const int b = __ffsll((long long)w) - 1;
                    float2 *cell = smh + (p * NH + __popcll(hmask & ((1ull << b) - 1ull))) * 256 + tid;
                    acc a = A::from2(*cell);
                    A::acc_add(a, bt[p]);
                    *cell = A::to2(a);
                }
            }
        }
        if (in_run)
#pragma unroll
            for (int p = 0; p < 2; ++p)
                cell_merge(p, run_hi, run[p]);
    }

    if (A::kRaises && bad)
        atomicOr(range_flag, 1);
    // deterministic reduction over the row lanes, NVB values a pass: in
    // double-float pairs on the float32 pipes (float64 only for the column
    // totals), or in float64 for the float64 accumulators
    if constexpr (A::kPairReduce)
    {
        float2 *rp = reinterpret_cast<float2 *>(red);
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
                    rp[w * 256 + tid] = A::to_pair(
                        i == 0 ? tot[p] : (i < 6 ? ml[p][i - 1] : A::from2(smh[(p * NH + i - 6) * 256 + tid])));
                }
            }
            __syncthreads();
            for (int s = TR >> 1; s > 0; s >>= 1)
            {
                if (tr < s)
#pragma unroll
                    for (int w = 0; w < NVB; ++w)
                    {
                        float2 x = rp[w * 256 + tid];
                        const float2 y = rp[w * 256 + tid + s * TC];
                        df_add(x.x, x.y, y.x, y.y);
                        rp[w * 256 + tid] = x;
                    }
                __syncthreads();
            }
            if (tr == 0)
#pragma unroll
                for (int w = 0; w < NVB; ++w)
                    if (v0 + w < NV)
                        res[(v0 + w) * TC + tc] = df_to_double(rp[w * 256 + tc].x, rp[w * 256 + tc].y);
            __syncthreads();
        }
    }
    else
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
                red[w * 256 + tid] = A::to_double(i == 0 ? tot[p]
                                                         : (i < 6 ? ml[p][i - 1]
                                                                  : A::from2(smh[(p * NH + i - 6) * 256 + tid])));
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

template <typename A, int NH, bool TAB>
cudaError_t launch_nh_tab(const void *psi, int64_t S, int n, const DevOp &op, const MargChunk *d_chunks,
                          int n_chunks, int TC, int n_ctiles, int n_splits, double *out, int *range_flag,
                          cudaStream_t st)
{
    constexpr int NV = 2 * (1 + 5 + NH);
    const size_t smem = (size_t)(8 * 256 + NV * TC) * sizeof(double) + (size_t)2 * NH * 256 * sizeof(float2);
    dim3 grid((unsigned)n_chunks, (unsigned)n_splits, (unsigned)n_ctiles);
    cudaError_t e =
        cudaFuncSetAttribute(k_expect_marg<A, NH, TAB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess)
        return e;
    k_expect_marg<A, NH, TAB><<<grid, 256, smem, st>>>((const typename A::in_t *)psi, S, n, op.recs, op.orig, op.P,
                                                       d_chunks, TC, n_splits, out, range_flag);
    return launched();
}

template <typename A, int NH>
cudaError_t launch_nh(const void *psi, int64_t S, int n, const DevOp &op, const MargChunk *d_chunks, int n_chunks,
                      int TC, int n_ctiles, int n_splits, double *out, int *range_flag, cudaStream_t st)
{
    // the offset table: the policies that use it, whole 32-row blocks, and
    // offsets 31 S that fit 32 bits
    if constexpr (A::kRowTable)
        if (n >= 5 && 32 * S < ((int64_t)1 << 31))
            return launch_nh_tab<A, NH, true>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out,
                                              range_flag, st);
    return launch_nh_tab<A, NH, false>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag,
                                       st);
}

template <int NH>
cudaError_t launch_marg_nh(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const MargChunk *d_chunks,
                           int n_chunks, int TC, int n_ctiles, int n_splits, double *out, int *range_flag,
                           const void *psi_df, cudaStream_t st)
{
    if (fp32)
        return launch_nh<ArF32, NH>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, nullptr, st);
    // df64 on the float32 pipes, then the float64 form for out-of-range inputs
    cudaError_t e =
        psi_df ? launch_nh<ArDFS, NH>(psi_df, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, nullptr, st)
               : launch_nh<ArDF, NH>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag, st);
    if (e != cudaSuccess)
        return e;
    return launch_nh<ArF64, NH>(psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag, st);
}

} // namespace

cudaError_t launch_expect_marg(bool fp32, const void *psi, int64_t S, int n, const DevOp &op,
                               const MargChunk *d_chunks, int n_chunks, int max_high_bits, int TC, int n_ctiles,
                               int n_splits, double *out, int *range_flag, const void *psi_df, cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    if (max_high_bits > kMargMaxHighBits)
        return cudaErrorInvalidValue;
    if (max_high_bits <= 9)
        return launch_marg_nh<9>(fp32, psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag,
                                 psi_df, st);
    return launch_marg_nh<18>(fp32, psi, S, n, op, d_chunks, n_chunks, TC, n_ctiles, n_splits, out, range_flag,
                              psi_df, st);
}

} // namespace fpg
