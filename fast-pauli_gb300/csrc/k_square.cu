// k_square.cu -- SummedPauliOp::square on the GPU.
//
// Replaces fast_pauli/cpp/include/__summed_pauli_op.hpp:197-268: for every
// operator k, A_k^2 = sum_{i,j} h(i,k) h(j,k) P_i P_j, with P_i P_j = phase *
// Q_a for a string Q_a of the squared set, so
//     out(a, k) = sum_{(i,j): P_i P_j ~ Q_a} phase(i,j) h(i,k) h(j,k).
// The reference builds the (i, j, phase) lists of every a on the host (P^2
// hash-map look-ups, serial) and contracts them with OpenMP.  Here:
//
//  * products are bit operations on the (x, z) encoding: P_i P_j has
//    x = x_i ^ x_j, z = z_i ^ z_j and phase i^e with
//        e = |x_i & z_i| + |x_j & z_j| - |x & z| + 2 |z_i & x_j|  (mod 4),
//    from sigma(x, z) = i^{xz} X^x Z^z per qubit and Z X = -X Z;
//  * the pairs of output string a are enumerated on the device (one warp per
//    a): for each i, the partners j are the strings with key (x_a ^ x_i,
//    z_a ^ z_i), found by binary search in the sorted encoding;
//  * h_i h_j is symmetric and P_j P_i = +-P_i P_j (commuting / anticommuting),
//    so only pairs with caller index j >= i that commute are kept, with
//    weight 2 (1 for i = j); anticommuting pairs cancel exactly.  That halves
//    the contraction and leaves a real phase (+-1) on every kept pair;
//  * the contraction out(a, k) runs output-stationary (one thread per (a, k),
//    k fastest, 8 k-lanes x 32 a-lanes per CTA) over a's pair list in a fixed
//    order, so results are deterministic; h rows stay in L1/L2.
//
// Strings of the squared set that occur twice take the products on their
// last occurrence (as the reference's index map, which keeps the last index
// inserted); a product missing from the set is counted as an error.
#include "common.cuh"

namespace fpg
{
namespace
{

struct SqTerm
{
    int32_t i, j; // caller indices
    int32_t e;    // phase exponent: phase = i^e
    int32_t w;    // 1 (i = j) or 2
};

__device__ __forceinline__ bool key_less(uint64_t x1, uint64_t z1, uint64_t x2, uint64_t z2)
{
    if (x1 != x2)
        return x1 < x2;
    const int p1 = __popcll(x1 & z1) & 1, p2 = __popcll(x2 & z2) & 1;
    if (p1 != p2)
        return p1 < p2;
    return z1 < z2;
}

// first sorted position whose (x, parity(#Y), z) key is not below (x, z)
__device__ __forceinline__ int lower_bound_key(const StringRec *__restrict__ recs, int P, uint64_t x, uint64_t z)
{
    int lo = 0, hi = P;
    while (lo < hi)
    {
        const int mid = (lo + hi) >> 1;
        if (key_less(recs[mid].x, recs[mid].z, x, z))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ bool commute(uint64_t xi, uint64_t zi, uint64_t xj, uint64_t zj)
{
    return ((__popcll(xi & zj) + __popcll(zi & xj)) & 1) == 0;
}

// Pass 1 (count) and pass 2 (fill) of the pair lists; one warp per sorted
// position sa of the squared set.
template <bool FILL>
__global__ void k_sq_pairs(const StringRec *__restrict__ a_recs, const int32_t *__restrict__ a_orig, int P,
                           const StringRec *__restrict__ q_recs, int A, int32_t *__restrict__ counts,
                           unsigned long long *__restrict__ n_found, const int64_t *__restrict__ offs,
                           SqTerm *__restrict__ terms)
{
    const int sa = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (sa >= A)
        return;
    const uint64_t xa = q_recs[sa].x, za = q_recs[sa].z;
    const bool dup = sa + 1 < A && q_recs[sa + 1].x == xa && q_recs[sa + 1].z == za;
    int kept = 0;
    unsigned long long found = 0;
    int64_t pos = FILL ? offs[sa] : 0;
    if (!dup)
    {
        const int na = __popcll(xa & za);
        for (int i0 = 0; i0 < P; i0 += 32)
        {
            const int i = i0 + lane;
            int c = 0, jb = 0, je = 0, oi = 0;
            uint64_t xi = 0, zi = 0, xj = 0, zj = 0;
            if (i < P)
            {
                xi = a_recs[i].x;
                zi = a_recs[i].z;
                xj = xa ^ xi;
                zj = za ^ zi;
                oi = a_orig[i];
                jb = lower_bound_key(a_recs, P, xj, zj);
                je = jb;
                while (je < P && a_recs[je].x == xj && a_recs[je].z == zj)
                    ++je;
                found += (unsigned long long)(je - jb);
                if (commute(xi, zi, xj, zj))
                    for (int j = jb; j < je; ++j)
                        c += a_orig[j] >= oi ? 1 : 0;
            }
            if (FILL)
            {
                // lanes write in i order: exclusive prefix of the lanes' counts
                int incl = c;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1)
                {
                    const int v = __shfl_up_sync(0xffffffffu, incl, d);
                    if (lane >= d)
                        incl += v;
                }
                int64_t w = pos + (incl - c);
                if (c)
                {
                    const int e =
                        (__popcll(xi & zi) + __popcll(xj & zj) - na + 2 * __popcll(zi & xj)) & 3;
                    for (int j = jb; j < je; ++j)
                    {
                        const int oj = a_orig[j];
                        if (oj >= oi)
                            terms[w++] = SqTerm{oi, oj, e, oj == oi ? 1 : 2};
                    }
                }
                pos += __shfl_sync(0xffffffffu, incl, 31);
            }
            kept += c;
        }
    }
    if (!FILL)
    {
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
        {
            kept += __shfl_xor_sync(0xffffffffu, kept, d);
            found += __shfl_xor_sync(0xffffffffu, found, d);
        }
        if (lane == 0)
        {
            counts[sa] = kept;
            atomicAdd(n_found, found);
        }
    }
}

// offs[a] = sum of counts[0 .. a), offs[A] = total; one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) k_sq_scan(const int32_t *__restrict__ counts, int A, int64_t *__restrict__ offs)
{
    __shared__ int64_t part[1024];
    const int t = threadIdx.x;
    const int per = (A + 1023) / 1024;
    const int b = min(A, t * per), e = min(A, b + per);
    int64_t s = 0;
    for (int k = b; k < e; ++k)
        s += counts[k];
    part[t] = s;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1)
    {
        const int64_t v = t >= d ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int64_t run = t ? part[t - 1] : 0;
    for (int k = b; k < e; ++k)
    {
        offs[k] = run;
        run += counts[k];
    }
    if (t == 1023)
        offs[A] = part[1023];
}

template <typename T> struct C2;
template <> struct C2<double>
{
    using type = double2;
};
template <> struct C2<float>
{
    using type = float2;
};

// out(orig_q[sa], k) = sum_terms w * i^e * h(i, k) h(j, k); every row written.
template <typename T>
__global__ void __launch_bounds__(256)
    k_sq_contract(const SqTerm *__restrict__ terms, const int64_t *__restrict__ offs,
                  const int32_t *__restrict__ q_orig, int A, const typename C2<T>::type *__restrict__ h, int64_t K,
                  typename C2<T>::type *__restrict__ out)
{
    using CT = typename C2<T>::type;
    const int kl = threadIdx.x & 7, al = threadIdx.x >> 3;
    const int64_t k = (int64_t)blockIdx.x * 8 + kl;
    if (k >= K)
        return;
    for (int64_t sa = (int64_t)blockIdx.y * 32 + al; sa < A; sa += (int64_t)gridDim.y * 32)
    {
        T re = T(0), im = T(0);
        const int64_t e1 = offs[sa + 1];
        for (int64_t e = offs[sa]; e < e1; ++e)
        {
            const SqTerm t = terms[e];
            const CT hi = __ldg(h + (int64_t)t.i * K + k);
            const CT hj = __ldg(h + (int64_t)t.j * K + k);
            // kept pairs commute: the phase is real, i^e = +-1 (e = 0 or 2)
            const T c = (t.e & 2) ? T(-t.w) : T(t.w);
            const T ar = c * hi.x, ai = c * hi.y;
            re = fma(ar, hj.x, re);
            re = fma(-ai, hj.y, re);
            im = fma(ar, hj.y, im);
            im = fma(ai, hj.x, im);
        }
        CT o;
        o.x = re;
        o.y = im;
        out[(int64_t)q_orig[sa] * K + k] = o;
    }
}

size_t align256(size_t b)
{
    return (b + 255) & ~(size_t)255;
}

} // namespace

int64_t square_max_terms(int64_t P)
{
    return P * (P + 1) / 2;
}

size_t square_workspace_bytes(int64_t P, int64_t A)
{
    return align256((size_t)A * 4) + align256((size_t)(A + 1) * 8) + align256(8) +
           align256((size_t)square_max_terms(P) * sizeof(SqTerm));
}

cudaError_t launch_square(bool fp32, const DevOp &op, const DevOp &sq, const void *h, int64_t K, void *out,
                          void *ws, unsigned long long **found, cudaStream_t st)
{
    const int P = (int)op.P, A = (int)sq.P;
    char *w = (char *)ws;
    int32_t *counts = (int32_t *)w;
    w += align256((size_t)A * 4);
    int64_t *offs = (int64_t *)w;
    w += align256((size_t)(A + 1) * 8);
    unsigned long long *n_found = (unsigned long long *)w;
    w += align256(8);
    SqTerm *terms = (SqTerm *)w;
    *found = n_found;
    cudaError_t e = cudaMemsetAsync(n_found, 0, 8, st);
    if (e != cudaSuccess)
        return e;
    const unsigned warps_per_cta = 8;
    const unsigned grid = (unsigned)((A + warps_per_cta - 1) / warps_per_cta);
    k_sq_pairs<false><<<grid, 32 * warps_per_cta, 0, st>>>(op.recs, op.orig, P, sq.recs, A, counts, n_found, nullptr,
                                                            nullptr);
    if ((e = launched()) != cudaSuccess)
        return e;
    k_sq_scan<<<1, 1024, 0, st>>>(counts, A, offs);
    if ((e = launched()) != cudaSuccess)
        return e;
    k_sq_pairs<true><<<grid, 32 * warps_per_cta, 0, st>>>(op.recs, op.orig, P, sq.recs, A, nullptr, nullptr, offs,
                                                           terms);
    if ((e = launched()) != cudaSuccess)
        return e;
    if (K <= 0)
        return cudaSuccess;
    const int64_t ay = (A + 31) / 32;
    dim3 cg((unsigned)((K + 7) / 8), (unsigned)(ay < 65535 ? ay : 65535));
    if (fp32)
        k_sq_contract<float><<<cg, 256, 0, st>>>(terms, offs, sq.orig, A, (const float2 *)h, K, (float2 *)out);
    else
        k_sq_contract<double><<<cg, 256, 0, st>>>(terms, offs, sq.orig, A, (const double2 *)h, K, (double2 *)out);
    return launched();
}

} // namespace fpg
