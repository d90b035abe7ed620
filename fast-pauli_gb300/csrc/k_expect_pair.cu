// k_expect_pair.cu -- per-string expectation values for x-groups whose sign
// patterns depend on at most one row bit.
//
// Same quantity as k_expect.cu (the per-string stage of
// SummedPauliOp::expectation_value, fast_pauli/cpp/include/__summed_pauli_op.hpp:572-577).
// For a group with x != 0 the rows i with the top bit p of x clear are
// paired with i ^ x (each pair counts twice, Pauli strings being Hermitian);
// a string's sign on those rows is (-1)^popc(i & z') with z' = z without
// bit p.  When every string of the group has z' in {0, e_a}
// for one bit a (e.g. the four strings XX, XY, YX, YY on two qubits), all of
// them are combinations of four sums,
//     U_c^re = sum_{i: bit a of i = c} Re q(i),  U_c^im likewise with Im q,
// W(0) = U_0 + U_1 and W(e_a) = U_0 - U_1, and the sums are accumulated with
// fused multiply-adds straight from the amplitudes:
//     U^re += a_r b_r + a_i b_i,  U^im += a_r b_i - a_i b_r
// -- four FMAs per row pair for the whole group, against q (4 operations)
// plus one signed add per string (4 more) in the direct kernel.  The x = 0
// group (diagonal strings) is summed over all rows.
//
// Layout as k_expect.cu: TC column lanes (V elements each) x (256 / TC) row
// lanes, 32-row blocks, grid (chunks, row splits, column tiles).  For
// x >= 32 whole blocks are paired (p >= 5); for 0 < x < 32 the pairs lie
// inside a block and only its 16 rows with bit p clear are visited.  Rows
// with bit a clear and set are visited side by side when a < 5; for a >= 5
// bit a is constant over a block.  float32: block sums in float32,
// Kahan-compensated across blocks, float64 across threads.
#include "df64.cuh"
#include "expect_body.cuh"

namespace fpg
{
namespace
{

template <typename T, int V>
__device__ __forceinline__ void fma_pair(const T (&ar)[V], const T (&ai)[V], const T (&br)[V], const T (&bi)[V],
                                         T (&sre)[V], T (&sim)[V])
{
#pragma unroll
    for (int v = 0; v < V; ++v)
    {
        sre[v] = fma(ar[v], br[v], fma(ai[v], bi[v], sre[v]));
        sim[v] = fma(ar[v], bi[v], fma(-ai[v], br[v], sim[v]));
    }
}

template <typename T> __device__ __forceinline__ void kahan_add(T &acc, T &cmp, T x)
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

// complex128 element -> df64 (re_h, re_l, im_h, im_l), integer ops only
// element e of the state: PRE = the df64 copy (float4 per element, split by
// k_df_split), else the complex128 state split here
template <bool PRE> __device__ __forceinline__ void load_df(const void *psi, int64_t e, float (&o)[4], bool &bad)
{
    float4 v;
    if constexpr (PRE)
        v = __ldg(reinterpret_cast<const float4 *>(psi) + e);
    else
        v = split_complex(__ldg(reinterpret_cast<const uint4 *>(psi) + e), bad);
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
}

// (re, im) += conj(a) b in df64: re += ar br + ai bi, im += ar bi - ai br
__device__ __forceinline__ void df_conj_mul_add(const float (&a)[4], const float (&b)[4], float (&re)[2],
                                                float (&im)[2])
{
    df_fma(a[0], a[1], b[0], b[1], re[0], re[1]);
    df_fma(a[2], a[3], b[2], b[3], re[0], re[1]);
    df_fma(a[0], a[1], b[2], b[3], im[0], im[1]);
    df_fma(-a[2], -a[3], b[0], b[1], im[0], im[1]);
}

// float64 path of the pair kernel on the float32 pipes: the same sums as
// k_expect_pair<double, 1> with every amplitude split into df64 (df64.cuh);
// df64 sums per 32-row block, df64 running sums across blocks, float64 only
// for the final cross-thread reduction.  Error <= ~2^-46 of sum |terms|.
// An amplitude outside the df64 range raises *range_flag (df64.cuh); with
// PRE the state comes split already (and checked) by k_df_split.
template <bool PRE, int V>
__global__ void __launch_bounds__(256, 2)
    k_expect_pair_df(const void *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                     const int32_t *__restrict__ orig, int64_t P, const PairChunk *__restrict__ chunks, int TC,
                     int n_splits, double *__restrict__ out, int *__restrict__ range_flag)
{
    static_assert(V == 1 || PRE, "two columns per thread read the split copy");
    // rows per load batch: four with one column, two with two (the same
    // bytes in flight, half the row-index work per column)
    constexpr int NB4 = V == 1 ? 4 : 2;
    bool bad = false;
    extern __shared__ double red[]; // blockDim.x * V doubles
    const PairChunk ch = chunks[blockIdx.x];
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const int64_t t0 = ((int64_t)blockIdx.z * TC + tc) * V; // S % V == 0
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
    const int abit = ch.abit;
    const bool split_in_block = abit >= 0 && abit < 5;
    const int e1 = split_in_block && pl >= 0 ? min(abit, pl) : (split_in_block ? abit : pl);
    const int e2 = split_in_block && pl >= 0 ? max(abit, pl) : -1;
    const int n_rows = 32 >> ((e1 >= 0) + (e2 >= 0));

    // running df64 sums [column][c][h/l]: U_c^re, U_c^im
    float ure[V][2][2], uim[V][2][2];
#pragma unroll
    for (int v = 0; v < V; ++v)
#pragma unroll
        for (int c = 0; c < 2; ++c)
            ure[v][c][0] = ure[v][c][1] = uim[v][c][0] = uim[v][c][1] = 0.f;
    if (col_ok)
    {
        for (int64_t m = b0 + tr; m < b1; m += TR)
        {
            const uint64_t um = (uint64_t)m;
            const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
            const uint64_t base = beta << 5;
            const uint64_t baseB = base ^ xh;
            float sre[V][2][2], sim[V][2][2];
#pragma unroll
            for (int v = 0; v < V; ++v)
#pragma unroll
                for (int c = 0; c < 2; ++c)
                    sre[v][c][0] = sre[v][c][1] = sim[v][c][0] = sim[v][c][1] = 0.f;
            // NB4 visited rows at a time, all their loads issued before any
            // use (the kernel is bound by L2 latency); n_rows is 8, 16 or 32
            for (int m0 = 0; m0 < n_rows; m0 += NB4)
            {
                uint32_t r0[NB4];
                bool ok[NB4];
#pragma unroll
                for (int u = 0; u < NB4; ++u)
                {
                    uint32_t r = (uint32_t)(m0 + u);
                    if (e1 >= 0)
                        r = ((r >> e1) << (e1 + 1)) | (r & ((1u << e1) - 1u));
                    if (e2 >= 0)
                        r = ((r >> e2) << (e2 + 1)) | (r & ((1u << e2) - 1u));
                    r0[u] = r;
                    ok[u] = (int)r < RB;
                }
                float a[NB4][V][4], b[NB4][V][4];
#pragma unroll
                for (int u = 0; u < NB4; ++u)
                    if (ok[u])
                    {
                        const int64_t ea = (int64_t)(base + r0[u]) * S + t0;
                        const int64_t eb = (int64_t)(baseB + (r0[u] ^ xl)) * S + t0;
#pragma unroll
                        for (int v = 0; v < V; ++v)
                        {
                            load_df<PRE>(psi, ea + v, a[u][v], bad);
                            load_df<PRE>(psi, eb + v, b[u][v], bad);
                        }
                    }
                if (split_in_block)
                {
                    // rows r1 = r0 | 2^a (< RB as a < n)
                    float c[NB4][V][4], d[NB4][V][4];
#pragma unroll
                    for (int u = 0; u < NB4; ++u)
                        if (ok[u])
                        {
                            const uint32_t r1 = r0[u] | (1u << abit);
                            const int64_t ec = (int64_t)(base + r1) * S + t0;
                            const int64_t ed = (int64_t)(baseB + (r1 ^ xl)) * S + t0;
#pragma unroll
                            for (int v = 0; v < V; ++v)
                            {
                                load_df<PRE>(psi, ec + v, c[u][v], bad);
                                load_df<PRE>(psi, ed + v, d[u][v], bad);
                            }
                        }
#pragma unroll
                    for (int u = 0; u < NB4; ++u)
                        if (ok[u])
#pragma unroll
                            for (int v = 0; v < V; ++v)
                                df_conj_mul_add(c[u][v], d[u][v], sre[v][1], sim[v][1]);
                }
#pragma unroll
                for (int u = 0; u < NB4; ++u)
                    if (ok[u])
#pragma unroll
                        for (int v = 0; v < V; ++v)
                            df_conj_mul_add(a[u][v], b[u][v], sre[v][0], sim[v][0]);
            }
            const int c0 = (abit >= 5) ? (int)((base >> abit) & 1u) : 0;
#pragma unroll
            for (int v = 0; v < V; ++v)
            {
                df_add(ure[v][c0][0], ure[v][c0][1], sre[v][0][0], sre[v][0][1]);
                df_add(uim[v][c0][0], uim[v][c0][1], sim[v][0][0], sim[v][0][1]);
                if (split_in_block)
                {
                    df_add(ure[v][1][0], ure[v][1][1], sre[v][1][0], sre[v][1][1]);
                    df_add(uim[v][1][0], uim[v][1][1], sim[v][1][0], sim[v][1][1]);
                }
            }
        }
    }

    if (!PRE && bad)
        atomicOr(range_flag, 1);
    // float64 reduction of the four sums over the row lanes (fixed order)
    double tot[4][V];
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            const float *u = q == 0 ? ure[v][0] : q == 1 ? ure[v][1] : q == 2 ? uim[v][0] : uim[v][1];
            red[(tr * TC + tc) * V + v] = df_to_double(u[0], u[1]);
        }
        __syncthreads();
        for (int s = TR >> 1; s > 0; s >>= 1)
        {
            if (tr < s)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    red[(tr * TC + tc) * V + v] += red[((tr + s) * TC + tc) * V + v];
            __syncthreads();
        }
#pragma unroll
        for (int v = 0; v < V; ++v)
            tot[q][v] = red[tc * V + v];
        __syncthreads();
    }
    if (tr != 0 || !col_ok)
        return;
    const uint64_t pbit = paired ? (1ull << (hb + 5)) : (pl >= 0 ? (1ull << pl) : 0ull);
    for (int k = 0; k < ch.count; ++k)
    {
        const int sidx = ch.begin + k;
        const StringRec rec = recs[sidx];
        const bool odd = (rec.meta & 1u) != 0;
        const bool flip = ((rec.z & ~pbit) != 0);
        const int ny = (int)(rec.meta & 3u);
        const double f = ((ny & 2) ? -1.0 : 1.0) * (pbit ? 2.0 : 1.0);
        double *dst = out + ((int64_t)blockIdx.y * P + orig[sidx]) * S + t0;
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            const double u0 = odd ? tot[2][v] : tot[0][v];
            const double u1 = odd ? tot[3][v] : tot[1][v];
            dst[v] = f * (flip ? u0 - u1 : u0 + u1);
        }
    }
}

// float32: residency for the latency-bound loads (V = 2 needs the registers
// of its four-row batches: two CTAs per SM)
template <typename T, int V> constexpr int kPairMinBlocks = sizeof(T) == 4 ? (V == 2 ? 2 : 3) : 1;

// only_if: when not null, the launch is the float64 recomputation after the
// df64 kernel and returns at once unless *only_if is set.
template <typename T, int V>
__global__ void __launch_bounds__(256, kPairMinBlocks<T, V>)
    k_expect_pair(const T *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                  const int32_t *__restrict__ orig, int64_t P, const PairChunk *__restrict__ chunks, int TC,
                  int n_splits, double *__restrict__ out, const int *__restrict__ only_if)
{
    if (only_if && *only_if == 0)
        return;
    extern __shared__ double red[]; // blockDim.x * V doubles
    const PairChunk ch = chunks[blockIdx.x];
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const int64_t t0 = ((int64_t)blockIdx.z * TC + tc) * V;
    const bool col_ok = t0 < S;

    const uint64_t D = 1ull << n;
    const uint64_t xh = ch.x & ~31ull;
    const uint32_t xl = (uint32_t)ch.x & 31u;
    const bool paired = xh != 0;                                // blocks paired
    const int pl = (!paired && xl != 0u) ? (31 - __clz((int)xl)) : -1; // rows paired inside a block
    const int64_t NB = n >= 5 ? (int64_t)(D >> 5) : 1;
    const int RB = n >= 5 ? 32 : (int)D;
    const int64_t nblk = paired ? NB / 2 : NB;
    const int hb = paired ? (63 - __clzll((long long)(xh >> 5))) : 0;
    const int64_t per = (nblk + n_splits - 1) / n_splits;
    const int64_t b0 = (int64_t)blockIdx.y * per;
    const int64_t b1 = min(nblk, b0 + per);
    const int abit = ch.abit; // -1: every string has z' = 0
    const bool split_in_block = abit >= 0 && abit < 5;
    // rows of a block visited: insert zero bits at pl and (a < 5) at a into
    // m = 0 .. 2^free - 1, lower excluded bit first
    const int e1 = split_in_block && pl >= 0 ? min(abit, pl) : (split_in_block ? abit : pl);
    const int e2 = split_in_block && pl >= 0 ? max(abit, pl) : -1;
    const int n_rows = 32 >> ((e1 >= 0) + (e2 >= 0));

    // accumulators [c][v]: U_c^re, U_c^im with Kahan compensation (float32)
    T ure[2][V], uim[2][V], cre[2][V], cim[2][V];
#pragma unroll
    for (int c = 0; c < 2; ++c)
#pragma unroll
        for (int v = 0; v < V; ++v)
            ure[c][v] = uim[c][v] = cre[c][v] = cim[c][v] = T(0);

    if (col_ok)
    {
        for (int64_t m = b0 + tr; m < b1; m += TR)
        {
            const uint64_t um = (uint64_t)m;
            const uint64_t beta = paired ? (((um >> hb) << (hb + 1)) | (um & ((1ull << hb) - 1ull))) : um;
            const uint64_t base = beta << 5;
            const uint64_t baseB = base ^ xh;
            T sre[2][V], sim[2][V];
#pragma unroll
            for (int c = 0; c < 2; ++c)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    sre[c][v] = sim[c][v] = T(0);
            // four visited rows at a time, all loads issued before any use
            // (L2-latency bound); n_rows is 8, 16 or 32
            for (int m0 = 0; m0 < n_rows; m0 += 4)
            {
                uint32_t r0[4];
                bool ok[4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                {
                    uint32_t r = (uint32_t)(m0 + u);
                    if (e1 >= 0)
                        r = ((r >> e1) << (e1 + 1)) | (r & ((1u << e1) - 1u));
                    if (e2 >= 0)
                        r = ((r >> e2) << (e2 + 1)) | (r & ((1u << e2) - 1u));
                    r0[u] = r;
                    ok[u] = (int)r < RB;
                }
                T ar[4][V], ai[4][V], br[4][V], bi[4][V];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (ok[u])
                    {
                        load_cvec<T, V>(psi + 2 * ((int64_t)(base + r0[u]) * S + t0), ar[u], ai[u]);
                        load_cvec<T, V>(psi + 2 * ((int64_t)(baseB + (r0[u] ^ xl)) * S + t0), br[u], bi[u]);
                    }
                if (split_in_block)
                {
                    // rows r1 = r0 | 2^a (< RB as a < n)
                    T cr[4][V], ci[4][V], dr[4][V], di[4][V];
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (ok[u])
                        {
                            const uint32_t r1 = r0[u] | (1u << abit);
                            load_cvec<T, V>(psi + 2 * ((int64_t)(base + r1) * S + t0), cr[u], ci[u]);
                            load_cvec<T, V>(psi + 2 * ((int64_t)(baseB + (r1 ^ xl)) * S + t0), dr[u], di[u]);
                        }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (ok[u])
                            fma_pair<T, V>(cr[u], ci[u], dr[u], di[u], sre[1], sim[1]);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (ok[u])
                        fma_pair<T, V>(ar[u], ai[u], br[u], bi[u], sre[0], sim[0]);
            }
            // block sums into the running sums: bit a of the block base picks
            // the accumulator when a >= 5
            const int c0 = (abit >= 5) ? (int)((base >> abit) & 1u) : 0;
#pragma unroll
            for (int v = 0; v < V; ++v)
            {
                if (c0 == 0)
                {
                    kahan_add(ure[0][v], cre[0][v], sre[0][v]);
                    kahan_add(uim[0][v], cim[0][v], sim[0][v]);
                }
                else
                {
                    kahan_add(ure[1][v], cre[1][v], sre[0][v]);
                    kahan_add(uim[1][v], cim[1][v], sim[0][v]);
                }
                if (split_in_block)
                {
                    kahan_add(ure[1][v], cre[1][v], sre[1][v]);
                    kahan_add(uim[1][v], cim[1][v], sim[1][v]);
                }
            }
        }
    }

    // reduce the four sums over the row lanes (float64, fixed order), then
    // thread row 0 writes every string of the chunk
    const int W = TC * V;
    double tot[4][V];
#pragma unroll
    for (int q = 0; q < 4; ++q)
    {
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            const T a = q == 0 ? ure[0][v] : q == 1 ? ure[1][v] : q == 2 ? uim[0][v] : uim[1][v];
            const T c = q == 0 ? cre[0][v] : q == 1 ? cre[1][v] : q == 2 ? cim[0][v] : cim[1][v];
            red[tr * W + tc * V + v] = (double)a - (double)c;
        }
        __syncthreads();
        for (int s = TR >> 1; s > 0; s >>= 1)
        {
            if (tr < s)
#pragma unroll
                for (int v = 0; v < V; ++v)
                    red[tr * W + tc * V + v] += red[(tr + s) * W + tc * V + v];
            __syncthreads();
        }
#pragma unroll
        for (int v = 0; v < V; ++v)
            tot[q][v] = red[tc * V + v];
        __syncthreads();
    }
    if (tr != 0 || !col_ok)
        return;
    const uint64_t pbit = paired ? (1ull << (hb + 5)) : (pl >= 0 ? (1ull << pl) : 0ull); // top bit of x
    for (int k = 0; k < ch.count; ++k)
    {
        const int sidx = ch.begin + k;
        const StringRec rec = recs[sidx];
        const bool odd = (rec.meta & 1u) != 0;
        const bool flip = ((rec.z & ~pbit) != 0); // z' = e_a
        const int ny = (int)(rec.meta & 3u);
        const double f = ((ny & 2) ? -1.0 : 1.0) * (pbit ? 2.0 : 1.0);
        double *dst = out + ((int64_t)blockIdx.y * P + orig[sidx]) * S + t0;
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            const double u0 = odd ? tot[2][v] : tot[0][v];
            const double u1 = odd ? tot[3][v] : tot[1][v];
            dst[v] = f * (flip ? u0 - u1 : u0 + u1);
        }
    }
}

} // namespace

cudaError_t launch_expect_pair(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const PairChunk *d_chunks,
                               int n_chunks, const ExpectPlan &plan, double *out, int *range_flag,
                               const void *psi_df, cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    dim3 grid((unsigned)n_chunks, (unsigned)plan.n_splits, (unsigned)plan.n_ctiles);
    const size_t smem = 256 * plan.V * sizeof(double);
    if (!fp32)
    {
        // df64 on the float32 pipes, then the float64 form for out-of-range
        // inputs.  With the split copy and an even number of states, two
        // adjacent columns per thread (half the column lanes, the same column
        // tile): half the row-index work per column.
        if (psi_df && S % 2 == 0 && plan.TC >= 2)
            k_expect_pair_df<true, 2><<<grid, 256, 2 * smem, st>>>(psi_df, S, n, op.recs, op.orig, op.P, d_chunks,
                                                                   plan.TC / 2, plan.n_splits, out, range_flag);
        else if (psi_df)
            k_expect_pair_df<true, 1><<<grid, 256, smem, st>>>(psi_df, S, n, op.recs, op.orig, op.P, d_chunks,
                                                               plan.TC, plan.n_splits, out, range_flag);
        else
            k_expect_pair_df<false, 1><<<grid, 256, smem, st>>>(psi, S, n, op.recs, op.orig, op.P, d_chunks, plan.TC,
                                                                plan.n_splits, out, range_flag);
        if (cudaError_t e = launched())
            return e;
        k_expect_pair<double, 1><<<grid, 256, smem, st>>>((const double *)psi, S, n, op.recs, op.orig, op.P, d_chunks,
                                                          plan.TC, plan.n_splits, out, range_flag);
    }
    else if (plan.V == 2)
        k_expect_pair<float, 2><<<grid, 256, smem, st>>>((const float *)psi, S, n, op.recs, op.orig, op.P, d_chunks,
                                                         plan.TC, plan.n_splits, out, nullptr);
    else
        k_expect_pair<float, 1><<<grid, 256, smem, st>>>((const float *)psi, S, n, op.recs, op.orig, op.P, d_chunks,
                                                         plan.TC, plan.n_splits, out, nullptr);
    return launched();
}

cudaError_t launch_expect_pair_f64_if(const void *psi, int64_t S, int n, const DevOp &op, const PairChunk *d_chunks,
                                      int n_chunks, const ExpectPlan &plan, double *out, const int *range_flag,
                                      cudaStream_t st)
{
    if (n_chunks <= 0)
        return cudaSuccess;
    dim3 grid((unsigned)n_chunks, (unsigned)plan.n_splits, (unsigned)plan.n_ctiles);
    k_expect_pair<double, 1><<<grid, 256, 256 * sizeof(double), st>>>(
        (const double *)psi, S, n, op.recs, op.orig, op.P, d_chunks, plan.TC, plan.n_splits, out, range_flag);
    return launched();
}

} // namespace fpg
