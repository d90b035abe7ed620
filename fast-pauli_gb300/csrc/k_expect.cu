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
// The chunk body lives in expect_body.cuh (shared with the batch kernel).
#include "expect_body.cuh"

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

// float32 chunks of up to four strings do little arithmetic per row and are
// bound by memory latency, so residency decides their speed: ask for three
// resident 256-thread CTAs per SM (<= 85 registers; measured 2.3x faster on
// uniform random strings at n = 20 than the 127-register default).
template <typename T, int G> constexpr int kExpectMinBlocks = (sizeof(T) == 4 && G <= 4) ? 3 : 1;

template <typename T, int V, int GE, int GO>
__global__ void __launch_bounds__(256, kExpectMinBlocks<T, GE + GO>)
    k_expect_chunks(const T *__restrict__ psi, int64_t S, int n, const StringRec *__restrict__ recs,
                    const int32_t *__restrict__ orig, int64_t P, const Chunk *__restrict__ chunks, int TC,
                    int n_splits, double *__restrict__ out)
{
    extern __shared__ double red[]; // blockDim.x * V doubles
    expect_chunk_body<T, V, GE, GO>(psi, S, n, recs, orig, P, chunks[blockIdx.x], TC, (int64_t)blockIdx.z,
                                    (int)blockIdx.y, n_splits, out, red);
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

__global__ void k_reduce_family(const double *__restrict__ partial, int n_splits, int64_t Pf, int64_t S,
                                const int32_t *__restrict__ glob, double *__restrict__ ev)
{
    const int64_t count = Pf * S;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < count; e += (int64_t)gridDim.x * blockDim.x)
    {
        double s = 0.0;
        for (int p = 0; p < n_splits; ++p)
            s += partial[(int64_t)p * count + e];
        const int64_t l = e / S;
        ev[(int64_t)glob[l] * S + (e - l * S)] = s;
    }
}

} // namespace

cudaError_t launch_reduce_family(const double *partial, int n_splits, int64_t Pf, int64_t S, const int32_t *glob,
                                 double *ev, cudaStream_t st)
{
    const int64_t count = Pf * S;
    if (count <= 0)
        return cudaSuccess;
    int64_t blocks = (count + 255) / 256;
    if (blocks > (int64_t)sm_count() * 16)
        blocks = (int64_t)sm_count() * 16;
    k_reduce_family<<<(unsigned)blocks, 256, 0, st>>>(partial, n_splits, Pf, S, glob, ev);
    return launched();
}

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

} // namespace fpg
