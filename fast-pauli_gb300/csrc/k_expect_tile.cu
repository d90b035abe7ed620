// k_expect_tile.cu -- per-string expectation values of the two-position
// x-groups, several groups per pass over the state.
//
// Same quantity as k_expect_pair.cu (the per-string stage of
// SummedPauliOp::expectation_value, fast_pauli/cpp/include/__summed_pauli_op.hpp:572-577)
// for the groups x = e_a + e_b (a < b) whose strings all have z' (z without
// bit b) in {0, e_a}: XX, XY, YX, YY on qubits a, b.  Each string is
// f (U_0 +- U_1) with U_c = sum over rows r with bit b clear and bit a = c of
// conj(psi_r) psi_{r ^ x}.
//
// The pair kernel reads the whole state once per group.  Here a work unit
// (TileChunk) is a set Q of four row bits q0 < q1 < q2 < q3 with up to six
// groups x = e_{q_i} + e_{q_j} (slot (i, j)): the rows split into 16-row
// tiles {base + sum_k t_k 2^{q_k}}, and every group of the unit pairs rows
// inside a tile.  A thread loads a tile's 16 rows of its column once and
// serves all six groups from registers: 16 loads for 48 row pairs instead
// of 96, and the row-index arithmetic once per tile.  Row t pairs with
// t ^ (2^i + 2^j) for t with bit j clear; c = bit i of t.
//
// Layout: TC column lanes (one complex element each) x TR = 256 / TC row
// lanes; grid (units, row splits, column tiles), units fastest, so that
// concurrent CTAs read the same column tile (sized to stay in L2).
// float32: tile sums in float32, Kahan-compensated across tiles.  float64:
// double-float (df64.cuh) on the float32 pipes from the split copy of the
// state (k_df_split): each tile's sums in offset accumulators (the offset a
// power of two above 16 times the tile's largest squared high part), their
// totals into running df64 sums; a value outside the df64 range was
// flagged by the split, and the pair kernel's float64 form recomputes the
// groups.  Both sum over the row lanes in double-float pairs and convert
// only the column totals to float64.
#include <type_traits>

#include "df64.cuh"
#include "expect_body.cuh"

namespace fpg
{
namespace
{

// slot s <-> the bit positions (i, j), i < j, of its group inside Q
__constant__ int8_t c_slot_j[kTileSlots] = {1, 2, 2, 3, 3, 3};
constexpr int kSlotI[kTileSlots] = {0, 0, 1, 0, 1, 2};
constexpr int kSlotJ[kTileSlots] = {1, 2, 2, 3, 3, 3};

template <typename T> __device__ __forceinline__ void tile_kahan(T &acc, T &cmp, T x)
{
    const T y = x - cmp;
    const T s = acc + y;
    cmp = (s - acc) - y;
    acc = s;
}

// Sums of NS slots: [slot][c][re, im].  df64 carries (hi, lo) pairs.
template <bool DF, int NS> struct TileAcc;

template <int NS> struct TileAcc<false, NS>
{
    float run[NS][2][2], cmp[NS][2][2];
    __device__ void zero()
    {
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
            for (int c = 0; c < 2; ++c)
                run[s][c][0] = run[s][c][1] = cmp[s][c][0] = cmp[s][c][1] = 0.f;
    }
    // the compensated sum as an unevaluated pair hi + lo
    __device__ float2 pair(int s, int c, int part) const
    {
        return make_float2(run[s][c][part], -cmp[s][c][part]);
    }
};

template <int NS> struct TileAcc<true, NS>
{
    float run[NS][2][2][2]; // [slot][c][re, im][hi, lo]
    __device__ void zero()
    {
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
            for (int c = 0; c < 2; ++c)
                run[s][c][0][0] = run[s][c][0][1] = run[s][c][1][0] = run[s][c][1][1] = 0.f;
    }
    __device__ float2 pair(int s, int c, int part) const
    {
        return make_float2(run[s][c][part][0], run[s][c][part][1]);
    }
    __device__ void norm()
    {
#pragma unroll
        for (int s = 0; s < NS; ++s)
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int p = 0; p < 2; ++p)
                    df_norm(run[s][c][p][0], run[s][c][p][1]);
    }
};

// one tile: rows[t] = the tile's row t of this thread's column.  float32:
// the four products of conj(a) b in separate sums per c (eight independent
// FMA chains per slot), combined once per tile
template <int S_>
__device__ __forceinline__ void tile_slot_f32(const float (&rows)[16][2], float (&ts)[2][2])
{
    constexpr int i = kSlotI[S_], j = kSlotJ[S_];
    float rr[2] = {0.f, 0.f}, ii[2] = {0.f, 0.f}, ri[2] = {0.f, 0.f}, ir[2] = {0.f, 0.f};
#pragma unroll
    for (int t = 0; t < 16; ++t)
        if (!((t >> j) & 1))
        {
            const int u = t ^ ((1 << i) | (1 << j));
            const int c = (t >> i) & 1;
            // conj(a) b: re = ar br + ai bi, im = ar bi - ai br
            rr[c] = fmaf(rows[t][0], rows[u][0], rr[c]);
            ii[c] = fmaf(rows[t][1], rows[u][1], ii[c]);
            ri[c] = fmaf(rows[t][0], rows[u][1], ri[c]);
            ir[c] = fmaf(-rows[t][1], rows[u][0], ir[c]);
        }
#pragma unroll
    for (int c = 0; c < 2; ++c)
    {
        ts[c][0] = rr[c] + ii[c];
        ts[c][1] = ri[c] + ir[c];
    }
}

// df64: each of the slot's four sums takes 8 products per tile, all bounded
// by m^2 (m = the largest high part of the tile's 16 rows), so the tile's
// sums run in offset accumulators (df_fma_offset, sigma = df_offset_for(m^2))
// and only their totals go through TwoSum into the running sums
template <int S_>
__device__ __forceinline__ void tile_slot_df(const float (&rows)[16][4], float sigma, float (&acc)[2][2][2])
{
    constexpr int i = kSlotI[S_], j = kSlotJ[S_];
    float h[2][2], l[2][2];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int p = 0; p < 2; ++p)
        {
            h[c][p] = sigma;
            l[c][p] = 0.f;
        }
#pragma unroll
    for (int t = 0; t < 16; ++t)
        if (!((t >> j) & 1))
        {
            const int u = t ^ ((1 << i) | (1 << j));
            const int c = (t >> i) & 1;
            const float(&a)[4] = rows[t];
            const float(&b)[4] = rows[u];
            df_fma_offset(a[0], a[1], b[0], b[1], h[c][0], l[c][0]);
            df_fma_offset(a[2], a[3], b[2], b[3], h[c][0], l[c][0]);
            df_fma_offset(a[0], a[1], b[2], b[3], h[c][1], l[c][1]);
            df_fma_offset(-a[2], -a[3], b[0], b[1], h[c][1], l[c][1]);
        }
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int p = 0; p < 2; ++p)
            df_add_lazy(acc[c][p][0], acc[c][p][1], __fsub_rn(h[c][p], sigma), l[c][p]);
}

// slot S_ of the unit into local accumulator L_, if active
template <int S_, int L_, int NS>
__device__ __forceinline__ void run_slot(const float (&rows)[16][2], TileAcc<false, NS> &A, int act)
{
    if (!((act >> L_) & 1))
        return;
    float ts[2][2];
    tile_slot_f32<S_>(rows, ts);
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int p = 0; p < 2; ++p)
            tile_kahan(A.run[L_][c][p], A.cmp[L_][c][p], ts[c][p]);
}

template <int S_, int L_, int NS>
__device__ __forceinline__ void run_slot(const float (&rows)[16][4], TileAcc<true, NS> &A, int act, float sigma)
{
    if (!((act >> L_) & 1))
        return;
    tile_slot_df<S_>(rows, sigma, A.run[L_]);
}

template <int S_, int L_, int NS>
__device__ __forceinline__ void run_slot(const float (&rows)[16][2], TileAcc<false, NS> &A, int act, float)
{
    run_slot<S_, L_>(rows, A, act);
}

// the NS slots of this CTA: all six, or the half sb / 3 (sigma: the df64
// tile offset, unused in float32)
template <int NS, typename Rows, typename Acc>
__device__ __forceinline__ void run_slots(const Rows &rows, Acc &A, int act, int sb, float sigma = 0.f)
{
    if constexpr (NS == kTileSlots)
    {
        run_slot<0, 0>(rows, A, act, sigma);
        run_slot<1, 1>(rows, A, act, sigma);
        run_slot<2, 2>(rows, A, act, sigma);
        run_slot<3, 3>(rows, A, act, sigma);
        run_slot<4, 4>(rows, A, act, sigma);
        run_slot<5, 5>(rows, A, act, sigma);
    }
    else if (sb == 0)
    {
        run_slot<0, 0>(rows, A, act, sigma);
        run_slot<1, 1>(rows, A, act, sigma);
        run_slot<2, 2>(rows, A, act, sigma);
    }
    else
    {
        run_slot<3, 0>(rows, A, act, sigma);
        run_slot<4, 1>(rows, A, act, sigma);
        run_slot<5, 2>(rows, A, act, sigma);
    }
}

template <bool DF, int NS> constexpr int kTileMinBlocks = DF ? (NS == kTileSlots ? 1 : 2) : (NS == kTileSlots ? 2 : 3);

// DF: psi = the df64 split copy (float4 per element); else float2 elements.
// NS = 6: one CTA per unit; NS = 3: two CTAs per unit (blockIdx.x = 2 unit +
// half), each with half the slots and half the accumulator registers.
// OFF32: 2^n x S < 2^31, so that the tile's first row and element index and
// the rows' offsets from it fit 32 bits (one wide multiply-add per row load)
template <bool DF, int NS, bool OFF32>
__global__ void __launch_bounds__(256, kTileMinBlocks<DF, NS>)
    k_expect_tile(const void *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                  const int32_t *__restrict__ orig, int64_t P, const TileChunk *__restrict__ units, int TC,
                  int n_splits, double *__restrict__ out)
{
    extern __shared__ double red[]; // 256 * 4 * NS float pairs, then TC * 4 * NS doubles
    using Off = std::conditional_t<OFF32, int32_t, int64_t>;
    __shared__ Off s_off[16];
    const TileChunk u = units[NS == kTileSlots ? blockIdx.x : blockIdx.x >> 1];
    const int sb = NS == kTileSlots ? 0 : (int)(blockIdx.x & 1) * NS; // first slot of this CTA
    int act = 0;
#pragma unroll
    for (int s = 0; s < NS; ++s)
        act |= (u.count[sb + s] > 0) ? (1 << s) : 0;
    if (act == 0)
        return; // a half without groups (uniform over the CTA)
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const int64_t t0 = (int64_t)blockIdx.z * TC + tc;
    const bool col_ok = t0 < S;
    const int q0 = u.q[0], q1 = u.q[1], q2 = u.q[2], q3 = u.q[3];
    if (tid < 16)
        s_off[tid] = (Off)(((uint64_t)(tid & 1) << q0) | ((uint64_t)((tid >> 1) & 1) << q1) |
                               ((uint64_t)((tid >> 2) & 1) << q2) | ((uint64_t)((tid >> 3) & 1) << q3)) *
                     S;
    __syncthreads();

    const int64_t nb = (int64_t)1 << (n - 4); // tiles
    const int64_t per = (nb + n_splits - 1) / n_splits;
    const int64_t b0 = (int64_t)blockIdx.y * per;
    const int64_t b1 = min(nb, b0 + per);

    TileAcc<DF, NS> A;
    A.zero();
    if (col_ok)
    {
        [[maybe_unused]] int since_norm = 0;
        for (int64_t m = b0 + tr; m < b1; m += TR)
        {
            // base: m with zero bits inserted at q0 < q1 < q2 < q3 (OFF32:
            // 2^n S < 2^31, so the row index and the element index fit 32 bits)
            int64_t e0;
            if constexpr (OFF32)
            {
                uint32_t b = (uint32_t)m;
                b = ((b >> q0) << (q0 + 1)) | (b & ((1u << q0) - 1u));
                b = ((b >> q1) << (q1 + 1)) | (b & ((1u << q1) - 1u));
                b = ((b >> q2) << (q2 + 1)) | (b & ((1u << q2) - 1u));
                b = ((b >> q3) << (q3 + 1)) | (b & ((1u << q3) - 1u));
                e0 = (int32_t)b * (int32_t)S + (int32_t)t0;
            }
            else
            {
                uint64_t base = (uint64_t)m;
                base = ((base >> q0) << (q0 + 1)) | (base & ((1ull << q0) - 1ull));
                base = ((base >> q1) << (q1 + 1)) | (base & ((1ull << q1) - 1ull));
                base = ((base >> q2) << (q2 + 1)) | (base & ((1ull << q2) - 1ull));
                base = ((base >> q3) << (q3 + 1)) | (base & ((1ull << q3) - 1ull));
                e0 = (int64_t)base * S + t0;
            }
            const float4 *row4 = reinterpret_cast<const float4 *>(psi) + e0;
            const float2 *row2 = reinterpret_cast<const float2 *>(psi) + e0;
            if constexpr (DF)
            {
                float rows[16][4];
                float m = 0.f; // largest high part of the tile
#pragma unroll
                for (int t = 0; t < 16; ++t)
                {
                    const float4 v = __ldg(row4 + s_off[t]);
                    rows[t][0] = v.x;
                    rows[t][1] = v.y;
                    rows[t][2] = v.z;
                    rows[t][3] = v.w;
                    m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.z)));
                }
                run_slots<NS>(rows, A, act, sb, df_offset_for(__fmul_rn(m, m)));
                // each running sum took one tile total: renormalise every 4 tiles
                if (++since_norm == 4)
                {
                    since_norm = 0;
                    A.norm();
                }
            }
            else
            {
                float rows[16][2];
#pragma unroll
                for (int t = 0; t < 16; ++t)
                {
                    const float2 v = __ldg(row2 + s_off[t]);
                    rows[t][0] = v.x;
                    rows[t][1] = v.y;
                }
                run_slots<NS>(rows, A, act, sb);
            }
        }
    }

    // the 4 x NS sums of every thread into shared memory as (hi, lo) float
    // pairs, summed over the row lanes in a fixed order (deterministic) in
    // double-float on the float32 pipes; only the column totals become
    // float64.  Then one thread per (column, slot) writes the slot's strings.
    constexpr int NQ = 4 * NS;
    float2 *pr = reinterpret_cast<float2 *>(red);
#pragma unroll
    for (int s = 0; s < NS; ++s)
#pragma unroll
        for (int c = 0; c < 2; ++c)
#pragma unroll
            for (int p = 0; p < 2; ++p)
                pr[(size_t)tid * NQ + s * 4 + p * 2 + c] = A.pair(s, c, p);
    __syncthreads();
    double *tots = red + (size_t)(TR * TC) * NQ / 2; // after the pairs
    for (int k = tid; k < TC * NQ; k += blockDim.x)
    {
        const int c = k / NQ, q = k - c * NQ;
        float h = 0.f, l = 0.f;
        for (int r = 0; r < TR; ++r)
        {
            const float2 v = pr[(size_t)(r * TC + c) * NQ + q];
            df_add(h, l, v.x, v.y);
        }
        tots[k] = df_to_double(h, l);
    }
    __syncthreads();
    if (tid >= TC * NS)
        return;
    const int c = tid % TC, ls = tid / TC, s = sb + ls;
    const int64_t col = (int64_t)blockIdx.z * TC + c;
    if (col >= S || u.count[s] == 0)
        return;
    const double *tot = tots + (size_t)c * NQ + ls * 4; // re c0, re c1, im c0, im c1
    const uint64_t pbit = 1ull << u.q[c_slot_j[s]];
    for (int k = 0; k < u.count[s]; ++k)
    {
        const int sidx = u.begin[s] + k;
        const StringRec rec = recs[sidx];
        const bool odd = (rec.meta & 1u) != 0;
        const bool flip = (rec.z & ~pbit) != 0; // z' = e_a
        const double f = ((rec.meta & 2u) ? -2.0 : 2.0);
        const double u0 = odd ? tot[2] : tot[0];
        const double u1 = odd ? tot[3] : tot[1];
        out[((int64_t)blockIdx.y * P + orig[sidx]) * S + col] = f * (flip ? u0 - u1 : u0 + u1);
    }
}

template <bool DF, int NS, bool OFF32>
cudaError_t launch_tile(const void *psi, int64_t S, int n, const DevOp &op, const TileChunk *d_units, int n_units,
                        int TC, int n_ctiles, int n_splits, double *out, cudaStream_t st)
{
    dim3 grid((unsigned)(n_units * (kTileSlots / NS)), (unsigned)n_splits, (unsigned)n_ctiles);
    // every thread's (hi, lo) pairs, then the column totals
    const size_t smem = (size_t)256 * 4 * NS * sizeof(float2) + (size_t)TC * 4 * NS * sizeof(double);
    if (cudaError_t e = cudaFuncSetAttribute(k_expect_tile<DF, NS, OFF32>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))
        return e;
    k_expect_tile<DF, NS, OFF32>
        <<<grid, 256, smem, st>>>(psi, S, n, op.recs, op.orig, op.P, d_units, TC, n_splits, out);
    return launched();
}

template <bool DF, int NS>
cudaError_t launch_tile(const void *psi, int64_t S, int n, const DevOp &op, const TileChunk *d_units, int n_units,
                        int TC, int n_ctiles, int n_splits, double *out, cudaStream_t st)
{
    // 32-bit row offsets and row index: the float64 step of the n=14
    // weight<=2 workload 2.92 -> 2.80 ms; the complex64 form at n=18 once
    // measured 8.5 -> 8.8 ms with 32-bit offsets alone, and 7.15 -> 7.09 ms
    // with the 32-bit row index added
    if ((((int64_t)1 << n) * S) < ((int64_t)1 << 31))
            return launch_tile<DF, NS, true>(psi, S, n, op, d_units, n_units, TC, n_ctiles, n_splits, out, st);
    return launch_tile<DF, NS, false>(psi, S, n, op, d_units, n_units, TC, n_ctiles, n_splits, out, st);
}

} // namespace

cudaError_t launch_expect_tile(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const TileChunk *d_units,
                               int n_units, int TC, int n_ctiles, int n_splits, double *out, cudaStream_t st)
{
    if (n_units <= 0)
        return cudaSuccess;
    // float32: one CTA per unit (128 registers, two CTAs per SM; halves, at
    // three CTAs per SM, ran 1.22x slower); float64: two CTAs per unit, so
    // that the accumulators of three slots fit two CTAs per SM (six slots
    // take 238 registers: one CTA per SM, 1.01x slower per step)
    if (fp32)
        return launch_tile<false, 6>(psi, S, n, op, d_units, n_units, TC, n_ctiles, n_splits, out, st);
    return launch_tile<true, 3>(psi, S, n, op, d_units, n_units, TC, n_ctiles, n_splits, out, st);
}

} // namespace fpg
