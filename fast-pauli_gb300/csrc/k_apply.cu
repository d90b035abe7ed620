// k_apply.cu -- apply kernels and their coefficient preparation, and the
// device sparse pattern.
//
// Replaces PauliString::apply_batch (fast_pauli/cpp/include/__pauli_string.hpp:378-436),
// PauliOp::apply (__pauli_op.hpp:399-468), SummedPauliOp::apply
// (__summed_pauli_op.hpp:277-349) and the per-string loop of
// SummedPauliOp::apply_weighted (__summed_pauli_op.hpp:441-455).
//
// With strings grouped by x, the operator is sum_g D_g X_g where X_g permutes
// rows (i -> i^x_g) and D_g is diagonal:
//     (D_g)_ii = sum_{j in g} c_j (-i)^{nY_j} (-1)^popc(i & z_j).
// Each output element is written once (no per-thread copies of the output as
// in the reference, __pauli_op.hpp:427): a thread owns (row i, V columns),
// walks the groups in a fixed order and accumulates
//     out(i,t) += sum_g (D_g)_ii psi(i^x_g, t).
// For apply_weighted the diagonal also depends on the column:
// w(j,t) (-i)^{nY_j} replaces c_j (-i)^{nY_j}.
#include "common.cuh"
#include "df64.cuh"

namespace fpg
{
namespace
{

template <typename T> struct C2;
template <> struct C2<double>
{
    using type = double2;
};
template <> struct C2<float>
{
    using type = float2;
};

// multiply by (-i)^ny
template <typename CT> __device__ __forceinline__ CT times_phase(CT c, int ny)
{
    CT r;
    switch (ny & 3)
    {
    case 0: r.x = c.x; r.y = c.y; break;
    case 1: r.x = c.y; r.y = -c.x; break;   // * (-i)
    case 2: r.x = -c.x; r.y = -c.y; break;  // * (-1)
    default: r.x = -c.y; r.y = c.x; break;  // * (+i)
    }
    return r;
}

template <typename CT>
__global__ void k_prep_coeffs(const StringRec *__restrict__ recs, const int32_t *__restrict__ orig, int64_t P,
                              const CT *__restrict__ coeffs, int64_t K, CT *__restrict__ cw)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P)
        return;
    const int64_t j = orig[s];
    CT c;
    if (K <= 0)
        c = coeffs[j];
    else
    {
        // row sum over operators, in the reference's order (__summed_pauli_op.hpp:312-317)
        c.x = 0;
        c.y = 0;
        for (int64_t k = 0; k < K; ++k)
        {
            const CT h = coeffs[j * K + k];
            c.x += h.x;
            c.y += h.y;
        }
    }
    cw[s] = times_phase(c, (int)(recs[s].meta & 3u));
}

template <typename CT>
__global__ void k_prep_weighted(const StringRec *__restrict__ recs, const int32_t *__restrict__ orig, int64_t P,
                                const CT *__restrict__ W, int64_t S, CT *__restrict__ cw)
{
    const int64_t total = P * S;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t s = e / S, t = e - s * S;
        cw[e] = times_phase(W[(int64_t)orig[s] * S + t], (int)(recs[s].meta & 3u));
    }
}

constexpr int kApplyRows = 8; // output rows per thread

// Bit k = parity(popcount((i0 + k) & z)) for the rows i0 .. i0+31 of a
// thread (i0 a multiple of the rows per thread, so all in one 32-row block):
// the string's parity table of the low five row bits, flipped by the parity
// of the high bits -- one popcount per string instead of one per row.
__device__ __forceinline__ uint32_t sign_bits(const StringRec &rec, uint64_t i0)
{
    const uint32_t hi = (uint32_t)(__popcll(i0 & rec.z & ~31ull) & 1);
    return (rec.mask_lo >> (uint32_t)(i0 & 31u)) ^ (0u - hi);
}

// (D_g)_ii of rows i0 .. i0+R-1 (one 32-row block) for column t: the group's
// coefficients, signed per row, summed in sorted string order from zero.
template <typename T, int R, bool WEIGHTED>
__device__ __forceinline__ void group_diag(const Group &gr, const StringRec *__restrict__ recs,
                                           const typename C2<T>::type *__restrict__ cw, int64_t S, int64_t t,
                                           uint64_t i0, T (&wr)[R], T (&wi)[R])
{
    using CT = typename C2<T>::type;
#pragma unroll
    for (int k = 0; k < R; ++k)
        wr[k] = wi[k] = T(0);
    for (int32_t s = gr.begin; s < gr.begin + gr.count; ++s)
    {
        const uint32_t sb = sign_bits(recs[s], i0);
        const CT c = WEIGHTED ? cw[(int64_t)s * S + t] : cw[s];
#pragma unroll
        for (int k = 0; k < R; ++k)
        {
            if ((sb >> k) & 1u)
            {
                wr[k] -= c.x;
                wi[k] -= c.y;
            }
            else
            {
                wr[k] += c.x;
                wi[k] += c.y;
            }
        }
    }
}

// The same in df64 from the coefficients' df64 copies (float4 per complex
// value): the first string's signed value, then a renormalised TwoSum per
// string.
template <int R, bool WEIGHTED>
__device__ __forceinline__ void group_diag_df(const Group &gr, const StringRec *__restrict__ recs,
                                              const float4 *__restrict__ cw, int64_t S, int64_t t, uint64_t i0,
                                              float (&wr)[R][2], float (&wi)[R][2])
{
    {
        const uint32_t sb = sign_bits(recs[gr.begin], i0);
        const float4 c = WEIGHTED ? cw[(int64_t)gr.begin * S + t] : cw[gr.begin];
#pragma unroll
        for (int k = 0; k < R; ++k)
        {
            const float sg = ((sb >> k) & 1u) ? -1.f : 1.f;
            wr[k][0] = sg * c.x;
            wr[k][1] = sg * c.y;
            wi[k][0] = sg * c.z;
            wi[k][1] = sg * c.w;
        }
    }
    for (int32_t s = gr.begin + 1; s < gr.begin + gr.count; ++s)
    {
        const uint32_t sb = sign_bits(recs[s], i0);
        const float4 c = WEIGHTED ? cw[(int64_t)s * S + t] : cw[s];
#pragma unroll
        for (int k = 0; k < R; ++k)
        {
            const float sg = ((sb >> k) & 1u) ? -1.f : 1.f;
            df_add(wr[k][0], wr[k][1], sg * c.x, sg * c.y);
            df_add(wi[k][0], wi[k][1], sg * c.z, sg * c.w);
        }
    }
}

// The same for rows i0 .. i0+3 (i0 a multiple of 4) by classes: row i0 + k
// differs from i0 only in bits 0..1, so (-1)^popc((i0 + k) & z) =
// (-1)^popc(i0 & z) (-1)^popc(k & z & 3).  Each string is added once, with
// its sign at i0, to the class of its z & 3 (A_0 .. A_3), and the rows'
// diagonals are the 4-point Walsh-Hadamard transform of the classes:
// (D_g)_{i0+k} = sum_c (-1)^popc(k & c) A_c.  Two df64 additions per string
// (and 16 per group) instead of eight; the class branch is uniform across a
// warp (every lane walks the same string).
template <bool WEIGHTED>
__device__ __forceinline__ void group_diag_df_classes(const Group &gr, const StringRec *__restrict__ recs,
                                                      const float4 *__restrict__ cw, int64_t S, int64_t t,
                                                      uint64_t i0, float (&wr)[4][2], float (&wi)[4][2])
{
    float ar[4][2], ai[4][2];
#pragma unroll
    for (int c = 0; c < 4; ++c)
        ar[c][0] = ar[c][1] = ai[c][0] = ai[c][1] = 0.f;
    for (int32_t s = gr.begin; s < gr.begin + gr.count; ++s)
    {
        const StringRec rec = recs[s];
        const float sg = (sign_bits(rec, i0) & 1u) ? -1.f : 1.f;
        const float4 c = WEIGHTED ? cw[(int64_t)s * S + t] : cw[s];
        const float xh = sg * c.x, xl = sg * c.y, yh = sg * c.z, yl = sg * c.w;
        switch ((uint32_t)rec.z & 3u)
        {
        case 0:
            df_add(ar[0][0], ar[0][1], xh, xl);
            df_add(ai[0][0], ai[0][1], yh, yl);
            break;
        case 1:
            df_add(ar[1][0], ar[1][1], xh, xl);
            df_add(ai[1][0], ai[1][1], yh, yl);
            break;
        case 2:
            df_add(ar[2][0], ar[2][1], xh, xl);
            df_add(ai[2][0], ai[2][1], yh, yl);
            break;
        default:
            df_add(ar[3][0], ar[3][1], xh, xl);
            df_add(ai[3][0], ai[3][1], yh, yl);
            break;
        }
    }
    // butterflies over class bit 0, then bit 1: u0 = A0 + A1, u1 = A0 - A1,
    // u2 = A2 + A3, u3 = A2 - A3; D0 = u0 + u2, D1 = u1 + u3, D2 = u0 - u2,
    // D3 = u1 - u3
    auto wht4 = [](float (&a)[4][2], float (&d)[4][2]) {
        float u[4][2];
#pragma unroll
        for (int h = 0; h < 2; ++h)
        {
            u[2 * h][0] = a[2 * h][0];
            u[2 * h][1] = a[2 * h][1];
            df_add(u[2 * h][0], u[2 * h][1], a[2 * h + 1][0], a[2 * h + 1][1]);
            u[2 * h + 1][0] = a[2 * h][0];
            u[2 * h + 1][1] = a[2 * h][1];
            df_add(u[2 * h + 1][0], u[2 * h + 1][1], -a[2 * h + 1][0], -a[2 * h + 1][1]);
        }
#pragma unroll
        for (int k = 0; k < 2; ++k)
        {
            d[k][0] = u[k][0];
            d[k][1] = u[k][1];
            df_add(d[k][0], d[k][1], u[k + 2][0], u[k + 2][1]);
            d[k + 2][0] = u[k][0];
            d[k + 2][1] = u[k][1];
            df_add(d[k + 2][0], d[k + 2][1], -u[k + 2][0], -u[k + 2][1]);
        }
    };
    wht4(ar, wr);
    wht4(ai, wi);
}

__device__ __forceinline__ float2 diag_entry(const Group &gr, const StringRec *__restrict__ recs,
                                             const float2 *__restrict__ cw, uint64_t i)
{
    float wr[1], wi[1];
    group_diag<float, 1, false>(gr, recs, cw, 1, 0, i, wr, wi);
    return make_float2(wr[0], wi[0]);
}

__device__ __forceinline__ float4 diag_entry(const Group &gr, const StringRec *__restrict__ recs,
                                             const float4 *__restrict__ cw, uint64_t i)
{
    float wr[1][2], wi[1][2];
    group_diag_df<1, false>(gr, recs, cw, 1, 0, i, wr, wi);
    return make_float4(wr[0][0], wr[0][1], wi[0][0], wi[0][1]);
}

// The group diagonals of a plain apply as a table diag[g * 2^n + i] =
// (D_g)_ii (float2: complex64 sums; float4: df64 sums): they do not depend
// on the column, so the apply kernels read them instead of summing each
// group's strings again in every column.  Each entry is summed by the same
// helper and in the same order as the in-register form, so both forms give
// the same bits.  Returns at once when *skip_if is set.
template <typename CT>
__global__ void k_group_diag(const Group *__restrict__ groups, int64_t G, const StringRec *__restrict__ recs,
                             const CT *__restrict__ cw, int n, CT *__restrict__ diag, const int *__restrict__ skip_if)
{
    if (skip_if && *skip_if)
        return;
    const uint64_t total = (uint64_t)G << n;
    const uint64_t rows = (1ull << n) - 1;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x)
        diag[e] = diag_entry(groups[e >> n], recs, cw, e & rows);
}

// only_if: when not null, the launch is the float64 form behind the df64
// kernel and returns at once unless *only_if is set.  TABLE: the group
// diagonals come from k_group_diag's table (plain apply only).
template <typename T, bool WEIGHTED, bool TABLE = false>
__global__ void __launch_bounds__(256)
    k_apply(const T *__restrict__ psi, T *__restrict__ out, int64_t S, int n, const Group *__restrict__ groups,
            int64_t G, const StringRec *__restrict__ recs, const typename C2<T>::type *__restrict__ cw, int TC,
            const int *__restrict__ only_if, const typename C2<T>::type *__restrict__ diag = nullptr)
{
    static_assert(!(TABLE && WEIGHTED), "the diagonal table holds column-independent diagonals");
    if (only_if && *only_if == 0)
        return;
    using CT = typename C2<T>::type;
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const uint64_t D = 1ull << n;
    // R consecutive rows per thread: the coefficients of a string (per column
    // for apply_weighted) are loaded once for all of them, and their partner
    // rows i ^ x_g lie side by side (R loads in flight per group)
    const uint64_t i0 = ((uint64_t)blockIdx.x * TR + tr) * kApplyRows;
    const int64_t t = (int64_t)blockIdx.y * TC + tc;
    if (i0 >= D || t >= S)
        return;
    const CT *ps = reinterpret_cast<const CT *>(psi);
    T accr[kApplyRows], acci[kApplyRows];
#pragma unroll
    for (int k = 0; k < kApplyRows; ++k)
        accr[k] = acci[k] = T(0);
    // groups in order, one at a time: every warp then sweeps the partner rows
    // i ^ x_g in step with its neighbours (loading several groups ahead per
    // thread measured 3x slower on large states: it scatters the reads)
    for (int64_t g = 0; g < G; ++g)
    {
        const Group gr = groups[g];
        CT b[kApplyRows];
#pragma unroll
        for (int k = 0; k < kApplyRows; ++k)
            if (i0 + k < D)
                b[k] = __ldg(ps + (int64_t)((i0 + k) ^ gr.x) * S + t);
        T wr[kApplyRows], wi[kApplyRows];
        if constexpr (TABLE)
        {
            const CT *dg = diag + (int64_t)g * (int64_t)D + (int64_t)i0;
#pragma unroll
            for (int k = 0; k < kApplyRows; ++k)
            {
                CT w;
                w.x = w.y = T(0);
                if (i0 + k < D)
                    w = __ldg(dg + k);
                wr[k] = w.x;
                wi[k] = w.y;
            }
        }
        else
            group_diag<T, kApplyRows, WEIGHTED>(gr, recs, cw, S, t, i0, wr, wi);
#pragma unroll
        for (int k = 0; k < kApplyRows; ++k)
            if (i0 + k < D)
            {
                accr[k] = fma(wr[k], b[k].x, fma(-wi[k], b[k].y, accr[k]));
                acci[k] = fma(wr[k], b[k].y, fma(wi[k], b[k].x, acci[k]));
            }
    }
#pragma unroll
    for (int k = 0; k < kApplyRows; ++k)
        if (i0 + k < D)
        {
            CT *o = reinterpret_cast<CT *>(out) + (int64_t)(i0 + k) * S + t;
            CT cur = *o;
            cur.x += accr[k];
            cur.y += acci[k];
            *o = cur;
        }
}

constexpr int kApplyRowsDf = 4; // output rows per thread, df64 form

// float64 apply in df64 on the float32 pipes (df64.cuh): the same sums as
// k_apply<double> with amplitudes and coefficients taken from their df64
// copies (float4 per complex value, split once per call); every product is
// exact (FMA error terms), every sum a TwoSum, the running sums are
// renormalised every 16 groups, and out += sum in float64 at the end.  Error
// ~2^-46 of sum |terms|.  Returns at once when *skip_if is set (an amplitude
// or coefficient outside the df64 range): k_apply<double> runs instead.
// TABLE: the group diagonals come from k_group_diag's table (plain apply).
// CLASSES: the diagonals of a thread's four rows from class sums
// (group_diag_df_classes): 2 df64 additions per string and 16 per group
// against 8 per string, so the launch picks it for operators with 3 or more
// strings per group on average (one kernel per choice: a per-group branch
// between both forms measured slower than either alone).
template <bool WEIGHTED, bool TABLE = false, bool CLASSES = false>
__global__ void __launch_bounds__(256)
    k_apply_df(const float4 *__restrict__ psi, double *__restrict__ out, int64_t S, int n,
               const Group *__restrict__ groups, int64_t G, const StringRec *__restrict__ recs,
               const float4 *__restrict__ cw, int TC, const int *__restrict__ skip_if,
               const float4 *__restrict__ diag = nullptr)
{
    static_assert(!(TABLE && WEIGHTED), "the diagonal table holds column-independent diagonals");
    static_assert(!(TABLE && CLASSES), "one source of diagonals");
    static_assert(!CLASSES || kApplyRowsDf == 4, "class sums cover four rows per thread");
    if (*skip_if)
        return;
    constexpr int R = kApplyRowsDf;
    const int tid = threadIdx.x;
    const int tc = tid & (TC - 1);
    const int tr = tid / TC;
    const int TR = blockDim.x / TC;
    const uint64_t D = 1ull << n;
    const uint64_t i0 = ((uint64_t)blockIdx.x * TR + tr) * R;
    const int64_t t = (int64_t)blockIdx.y * TC + tc;
    if (i0 >= D || t >= S)
        return;
    // running sums [row][h/l]
    float ar[R][2], ai[R][2];
#pragma unroll
    for (int k = 0; k < R; ++k)
        ar[k][0] = ar[k][1] = ai[k][0] = ai[k][1] = 0.f;
    for (int64_t g = 0; g < G; ++g)
    {
        const Group gr = groups[g];
        float4 b[R];
#pragma unroll
        for (int k = 0; k < R; ++k)
            b[k] = i0 + k < D ? __ldg(psi + (int64_t)((i0 + k) ^ gr.x) * S + t) : make_float4(0.f, 0.f, 0.f, 0.f);
        // diagonal of the group per row: sum of +-c over its strings (df64)
        float wr[R][2], wi[R][2];
        if constexpr (TABLE)
        {
            const float4 *dg = diag + (int64_t)g * (int64_t)D + (int64_t)i0;
#pragma unroll
            for (int k = 0; k < R; ++k)
            {
                const float4 w = i0 + k < D ? __ldg(dg + k) : make_float4(0.f, 0.f, 0.f, 0.f);
                wr[k][0] = w.x;
                wr[k][1] = w.y;
                wi[k][0] = w.z;
                wi[k][1] = w.w;
            }
        }
        else if constexpr (CLASSES)
            group_diag_df_classes<WEIGHTED>(gr, recs, cw, S, t, i0, wr, wi);
        else
            group_diag_df<R, WEIGHTED>(gr, recs, cw, S, t, i0, wr, wi);
        // sum += w * b  (complex, df64)
#pragma unroll
        for (int k = 0; k < R; ++k)
        {
            df_fma(wr[k][0], wr[k][1], b[k].x, b[k].y, ar[k][0], ar[k][1]);
            df_fma(-wi[k][0], -wi[k][1], b[k].z, b[k].w, ar[k][0], ar[k][1]);
            df_fma(wr[k][0], wr[k][1], b[k].z, b[k].w, ai[k][0], ai[k][1]);
            df_fma(wi[k][0], wi[k][1], b[k].x, b[k].y, ai[k][0], ai[k][1]);
        }
        if ((g & 15) == 15)
#pragma unroll
            for (int k = 0; k < R; ++k)
            {
                df_norm(ar[k][0], ar[k][1]);
                df_norm(ai[k][0], ai[k][1]);
            }
    }
#pragma unroll
    for (int k = 0; k < R; ++k)
        if (i0 + k < D)
        {
            double2 *o = reinterpret_cast<double2 *>(out) + (int64_t)(i0 + k) * S + t;
            double2 cur = *o;
            cur.x += df_to_double(ar[k][0], ar[k][1]);
            cur.y += df_to_double(ai[k][0], ai[k][1]);
            *o = cur;
        }
}

// out(k, i, i ^ x_g) += sum_{s in g} coeffs(orig[s], k) (-i)^nY_s (-1)^popc(i & z_s)
// for every operator k, row i and x-group g: each output element belongs to
// one (k, i, g), so the additions need no atomics.
template <typename CT>
__global__ void k_to_tensor(const StringRec *__restrict__ recs, const int32_t *__restrict__ orig,
                            const Group *__restrict__ groups, int64_t G, const CT *__restrict__ coeffs, int64_t K,
                            int n, CT *__restrict__ out)
{
    const uint64_t D = 1ull << n;
    const uint64_t total = (uint64_t)K * D * (uint64_t)G;
    for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (uint64_t)gridDim.x * blockDim.x)
    {
        const uint64_t i = e % D; // rows fastest: consecutive threads write neighbouring rows
        const uint64_t rest = e / D;
        const int64_t g = (int64_t)(rest % (uint64_t)G);
        const int64_t k = (int64_t)(rest / (uint64_t)G);
        const Group gr = groups[g];
        CT v;
        v.x = 0;
        v.y = 0;
        for (int32_t s = gr.begin; s < gr.begin + gr.count; ++s)
        {
            CT c = times_phase(coeffs[(int64_t)orig[s] * K + k], (int)(recs[s].meta & 3u));
            if (__popcll(i & recs[s].z) & 1)
            {
                c.x = -c.x;
                c.y = -c.y;
            }
            v.x += c.x;
            v.y += c.y;
        }
        CT &dst = out[((uint64_t)k * D + i) * D + (i ^ gr.x)];
        dst.x += v.x;
        dst.y += v.y;
    }
}

__global__ void k_sparse_repr(uint64_t x, uint64_t z, int ny, uint64_t D, uint64_t *__restrict__ cols,
                              double2 *__restrict__ vals)
{
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < D; i += (uint64_t)gridDim.x * blockDim.x)
    {
        cols[i] = i ^ x;
        double2 one = make_double2((__popcll(i & z) & 1) ? -1.0 : 1.0, 0.0);
        vals[i] = times_phase(one, ny);
    }
}

int pick_tc(int64_t S)
{
    int tc = 1;
    while (tc < 32 && tc < S)
        tc <<= 1;
    return tc;
}

} // namespace

cudaError_t launch_prep_coeffs(bool fp32, const DevOp &op, const void *coeffs, int64_t K, void *cw, cudaStream_t st)
{
    if (op.P <= 0)
        return cudaSuccess;
    const unsigned blocks = (unsigned)((op.P + 255) / 256);
    if (fp32)
        k_prep_coeffs<float2><<<blocks, 256, 0, st>>>(op.recs, op.orig, op.P, (const float2 *)coeffs, K,
                                                      (float2 *)cw);
    else
        k_prep_coeffs<double2><<<blocks, 256, 0, st>>>(op.recs, op.orig, op.P, (const double2 *)coeffs, K,
                                                       (double2 *)cw);
    return launched();
}

cudaError_t launch_prep_weighted(bool fp32, const DevOp &op, const void *W, int64_t S, void *cw, cudaStream_t st)
{
    if (op.P <= 0 || S <= 0)
        return cudaSuccess;
    int64_t blocks = (op.P * S + 255) / 256;
    if (blocks > (int64_t)sm_count() * 16)
        blocks = (int64_t)sm_count() * 16;
    const unsigned grid = (unsigned)blocks;
    if (fp32)
        k_prep_weighted<float2><<<grid, 256, 0, st>>>(op.recs, op.orig, op.P, (const float2 *)W, S, (float2 *)cw);
    else
        k_prep_weighted<double2><<<grid, 256, 0, st>>>(op.recs, op.orig, op.P, (const double2 *)W, S,
                                                       (double2 *)cw);
    return launched();
}

// Column lanes of an apply launch: up to 32, fewer while a column tile (all
// 2^n rows x TC columns, the rows the groups' partners i ^ x_g are gathered
// from) would not stay in L2 -- down to 64-byte row segments.  CTAs run in
// column-tile order, so the gathers of one tile then hit L2.
constexpr int64_t kApplyTileBytes = int64_t(48) << 20;
int apply_lanes(int64_t S, int n, int esz)
{
    int tc = pick_tc(S);
    while (tc * esz > 64 && ((int64_t(1) << n) * tc * esz) > kApplyTileBytes)
        tc >>= 1;
    return tc;
}

cudaError_t launch_group_diag(bool df, const DevOp &op, const void *cw, void *diag, const int *skip_if,
                              cudaStream_t st)
{
    if (op.G <= 0)
        return cudaSuccess;
    const uint64_t total = (uint64_t)op.G << op.n;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > (uint64_t)sm_count() * 16)
        blocks = (uint64_t)sm_count() * 16;
    if (df)
        k_group_diag<float4><<<(unsigned)blocks, 256, 0, st>>>(op.groups, op.G, op.recs, (const float4 *)cw, op.n,
                                                               (float4 *)diag, skip_if);
    else
        k_group_diag<float2><<<(unsigned)blocks, 256, 0, st>>>(op.groups, op.G, op.recs, (const float2 *)cw, op.n,
                                                               (float2 *)diag, skip_if);
    return launched();
}

cudaError_t launch_apply(bool fp32, bool weighted, const DevOp &op, const void *cw, const void *psi, void *out,
                         int64_t S, cudaStream_t st, const int *only_if, const void *diag)
{
    if (S <= 0 || op.G <= 0)
        return cudaSuccess;
    if (diag && (!fp32 || weighted))
        return cudaErrorInvalidValue;
    const int TC = apply_lanes(S, op.n, fp32 ? 8 : 16);
    const int TR = 256 / TC;
    const uint64_t D = 1ull << op.n;
    const uint64_t rows_per_cta = (uint64_t)TR * kApplyRows;
    dim3 grid((unsigned)((D + rows_per_cta - 1) / rows_per_cta), (unsigned)((S + TC - 1) / TC));
    if (fp32)
    {
        if (diag)
            k_apply<float, false, true><<<grid, 256, 0, st>>>((const float *)psi, (float *)out, S, op.n, op.groups,
                                                              op.G, op.recs, (const float2 *)cw, TC, only_if,
                                                              (const float2 *)diag);
        else if (weighted)
            k_apply<float, true><<<grid, 256, 0, st>>>((const float *)psi, (float *)out, S, op.n, op.groups, op.G,
                                                       op.recs, (const float2 *)cw, TC, only_if);
        else
            k_apply<float, false><<<grid, 256, 0, st>>>((const float *)psi, (float *)out, S, op.n, op.groups, op.G,
                                                        op.recs, (const float2 *)cw, TC, only_if);
    }
    else
    {
        if (weighted)
            k_apply<double, true><<<grid, 256, 0, st>>>((const double *)psi, (double *)out, S, op.n, op.groups, op.G,
                                                        op.recs, (const double2 *)cw, TC, only_if);
        else
            k_apply<double, false><<<grid, 256, 0, st>>>((const double *)psi, (double *)out, S, op.n, op.groups,
                                                         op.G, op.recs, (const double2 *)cw, TC, only_if);
    }
    return launched();
}

cudaError_t launch_apply_df(bool weighted, const DevOp &op, const void *cw_df, const void *psi_df, void *out,
                            int64_t S, const int *skip_if, cudaStream_t st, const void *diag)
{
    if (S <= 0 || op.G <= 0)
        return cudaSuccess;
    if (diag && weighted)
        return cudaErrorInvalidValue;
    const int TC = apply_lanes(S, op.n, 16);
    const int TR = 256 / TC;
    const uint64_t D = 1ull << op.n;
    const uint64_t rows_per_cta = (uint64_t)TR * kApplyRowsDf;
    dim3 grid((unsigned)((D + rows_per_cta - 1) / rows_per_cta), (unsigned)((S + TC - 1) / TC));
    if (diag)
        k_apply_df<false, true><<<grid, 256, 0, st>>>((const float4 *)psi_df, (double *)out, S, op.n, op.groups,
                                                      op.G, op.recs, (const float4 *)cw_df, TC, skip_if,
                                                      (const float4 *)diag);
    else if (weighted && op.P >= 3 * op.G)
        k_apply_df<true, false, true><<<grid, 256, 0, st>>>((const float4 *)psi_df, (double *)out, S, op.n,
                                                            op.groups, op.G, op.recs, (const float4 *)cw_df, TC,
                                                            skip_if);
    else if (weighted)
        k_apply_df<true><<<grid, 256, 0, st>>>((const float4 *)psi_df, (double *)out, S, op.n, op.groups, op.G,
                                               op.recs, (const float4 *)cw_df, TC, skip_if);
    else
        k_apply_df<false><<<grid, 256, 0, st>>>((const float4 *)psi_df, (double *)out, S, op.n, op.groups, op.G,
                                                op.recs, (const float4 *)cw_df, TC, skip_if);
    return launched();
}

cudaError_t launch_to_tensor(bool fp32, const DevOp &op, const void *coeffs, int64_t K, void *out, cudaStream_t st)
{
    if (K <= 0 || op.G <= 0)
        return cudaSuccess;
    const uint64_t total = (uint64_t)K * (1ull << op.n) * (uint64_t)op.G;
    uint64_t blocks = (total + 255) / 256;
    if (blocks > (int64_t)sm_count() * 32)
        blocks = (int64_t)sm_count() * 32;
    if (fp32)
        k_to_tensor<float2><<<(unsigned)blocks, 256, 0, st>>>(op.recs, op.orig, op.groups, op.G,
                                                              (const float2 *)coeffs, K, op.n, (float2 *)out);
    else
        k_to_tensor<double2><<<(unsigned)blocks, 256, 0, st>>>(op.recs, op.orig, op.groups, op.G,
                                                               (const double2 *)coeffs, K, op.n, (double2 *)out);
    return launched();
}

cudaError_t launch_sparse_repr(uint64_t x, uint64_t z, int ny, int n, uint64_t *cols, void *vals, cudaStream_t st)
{
    const uint64_t D = 1ull << n;
    uint64_t blocks = (D + 255) / 256;
    if (blocks > (int64_t)sm_count() * 32)
        blocks = (int64_t)sm_count() * 32;
    k_sparse_repr<<<(unsigned)blocks, 256, 0, st>>>(x, z, ny, D, cols, (double2 *)vals);
    return launched();
}

} // namespace fpg
