// k_contract_tc.cu -- 3xTF32 coefficient contraction on the 5th-generation
// tensor cores (tcgen05 + TMEM), for the mixed (complex64) path.
//
// Contraction of SummedPauliOp::expectation_value
// (fast_pauli/cpp/include/__summed_pauli_op.hpp:579-591) and the weighted
// coefficients of apply_weighted (__summed_pauli_op.hpp:420-432), both as a
// real GEMM  C(M,N) = A(M,Kd) B(N,Kd)^T  with float32 accumulation:
//   * expectation: A = [Re H^T; Im H^T] (2K x P), B = E^T (S x P), C (2K x S);
//   * apply_weighted: A = [Re H; Im H] (2P x K), B = X^T (S x K), C (2P x S).
// Split precision (3xTF32): every operand x = x_hi + x_lo with
// x_hi = tf32(x) (round to nearest) and x_lo = tf32(x - x_hi); the product is
// A_hi B_hi + A_hi B_lo + A_lo B_hi, accumulated in float32 in TMEM over one
// 32-deep k segment per CTA (grid z = segment); the finishing kernels sum the
// segments in double-float on the float32 pipes (TwoSum: ~2^-48 of the sum of
// their magnitudes, far below the complex64 output's rounding).  Long float32
// accumulations over thousands of terms
// with cancellation (e.g. a PauliOp with 4096 strings, K = 1) otherwise lose
// ~1e-5 relative accuracy.
//
// Data movement: a prep kernel writes each operand in the canonical K-major,
// no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix), one
// contiguous 16 KiB block per (128-row tile, 32-deep k chunk), so the GEMM
// moves blocks with 1-D TMA bulk copies (cp.async.bulk, completion on an
// mbarrier).  One elected thread issues copies and tcgen05.mma (M=128,
// N=128, K=8 per instruction, 3 per k step); tcgen05.commit signals stage
// reuse; a two-stage ring overlaps copies with MMAs.  The epilogue reads the
// 128x128 float32 accumulator with tcgen05.ld (warp w owns TMEM lanes
// 32w..32w+31) and writes a row-major float32 tile.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error code
// (fpg_device_error reports it), still waits (bounded) for its own copies and
// MMAs, frees its TMEM and returns.
#include <algorithm>
#include <cstdint>

#include "common.cuh"

namespace fpg
{

__device__ int g_tc_error = 0;

namespace
{

constexpr int TM = 128, TN = 128, TK = 32;           // CTA tile and k chunk (tf32 elements)
constexpr int BLOCK_BYTES = TM * TK * 4;             // 16 KiB per operand block
constexpr int STAGE_BYTES = 4 * BLOCK_BYTES;         // A_hi, A_lo, B_hi, B_lo
constexpr int NSTAGE = 2;
constexpr int SMEM_BYTES = NSTAGE * STAGE_BYTES + 2048; // + 1024-byte alignment pad, barriers, TMEM address
constexpr uint32_t TMEM_COLS = 128;
constexpr long long WAIT_LIMIT = 1ll << 22;          // mbarrier polls before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// bounded wait on phase `parity`; returns false on timeout
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity)
{
    const uint32_t a = smem_u32(bar);
    for (long long it = 0; it < WAIT_LIMIT; ++it)
    {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(a), "r"(parity)
                     : "memory");
        if (done)
            return true;
    }
    return false;
}

__device__ __forceinline__ void bulk_copy_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// Shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte
// offset >> 4 (16-29; K-direction stride between core matrices), stride byte
// offset >> 4 (32-45; stride between 8-row groups), descriptor version 1
// (bits 46-47), no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::tf32: D = f32 (bits 4-5 = 1), A = B = tf32
// (bits 7-9 and 10-12 = 2), both K-major, N >> 3 at bits 17-22, M >> 4 at
// bits 24-28.
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(TN >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
                 "l"(da), "l"(db), "r"(IDESC), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ float tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// byte offset of element (row r, k) inside a 128 x 32 operand block
__device__ __forceinline__ uint32_t block_offset(int r, int k)
{
    return (uint32_t)((r >> 3) * 1024 + (k >> 2) * 128 + (r & 7) * 16 + (k & 3) * 4);
}

// --------------------------------------------------------------- operand prep
// Writes hi/lo tf32 blocks for a rows x depth operand whose element (r, k) is
// produced by `load(r, k)` (zero outside the logical size).  Block index =
// row_tile * n_kchunks + kchunk.
template <typename Load>
__device__ void write_operand(Load load, int64_t rows, int64_t depth, int64_t rows_pad, int64_t depth_pad,
                              float *hi, float *lo)
{
    const int64_t kchunks = depth_pad / TK;
    const int64_t total = rows_pad * depth_pad;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t r = e / depth_pad, k = e - r * depth_pad;
        double v = (r < rows && k < depth) ? load(r, k) : 0.0;
        const float f = (float)v;
        const float h = tf32_rna(f);
        const float l = tf32_rna((float)(v - (double)h));
        const int64_t blk = (r / TM) * kchunks + (k / TK);
        const int64_t off = blk * (BLOCK_BYTES / 4) + block_offset((int)(r % TM), (int)(k % TK)) / 4;
        hi[off] = h;
        lo[off] = l;
    }
}

// expectation: A(m, p) = m < K ? Re H[p][m] : Im H[p][m-K];  H complex64 (P,K)
__global__ void k_prep_a_expect(const float2 *__restrict__ H, int64_t P, int64_t K, int64_t rows_pad,
                                int64_t depth_pad, float *hi, float *lo)
{
    write_operand(
        [&](int64_t m, int64_t p) -> double {
            const float2 h = H[p * K + (m < K ? m : m - K)];
            return m < K ? h.x : h.y;
        },
        2 * K, P, rows_pad, depth_pad, hi, lo);
}

// expectation: B(t, p) = E[p][t];  E float64 (P,S)
__global__ void k_prep_b_expect(const double *__restrict__ E, int64_t P, int64_t S, int64_t rows_pad,
                                int64_t depth_pad, float *hi, float *lo)
{
    write_operand([&](int64_t t, int64_t p) -> double { return E[p * S + t]; }, S, P, rows_pad, depth_pad, hi, lo);
}

// weighted: A(m, k) = m < P ? Re H[m][k] : Im H[m-P][k]
__global__ void k_prep_a_weighted(const float2 *__restrict__ H, int64_t P, int64_t K, int64_t rows_pad,
                                  int64_t depth_pad, float *hi, float *lo)
{
    write_operand(
        [&](int64_t m, int64_t k) -> double {
            const float2 h = H[(m < P ? m : m - P) * K + k];
            return m < P ? h.x : h.y;
        },
        2 * P, K, rows_pad, depth_pad, hi, lo);
}

// weighted: B(t, k) = X[k][t];  X float32 (K,S)
__global__ void k_prep_b_weighted(const float *__restrict__ X, int64_t K, int64_t S, int64_t rows_pad,
                                  int64_t depth_pad, float *hi, float *lo)
{
    write_operand([&](int64_t t, int64_t k) -> double { return X[k * S + t]; }, S, K, rows_pad, depth_pad, hi,
                  lo);
}

// ------------------------------------------------------------------- GEMM
// One 128x128 tile of one k segment per CTA (blockIdx.z = segment of
// seg_chunks 32-deep chunks): C[z] (rows_pad x cols_pad, row-major float32)
// = A B^T restricted to the segment.  Accumulation is float32 inside a
// segment only; the finishing kernels sum the segments in double-float.
__global__ void __launch_bounds__(128, 1)
    k_gemm_tf32x3(const float *__restrict__ a_hi, const float *__restrict__ a_lo, const float *__restrict__ b_hi,
                  const float *__restrict__ b_lo, int64_t kchunks, int64_t seg_chunks, int64_t rows_pad,
                  int64_t cols_pad, float *__restrict__ C)
{
    const int64_t kb = (int64_t)blockIdx.z * seg_chunks;
    const int64_t nk = min(kchunks, kb + seg_chunks) - kb; // chunks of this segment (>= 1)
    C += (int64_t)blockIdx.z * rows_pad * cols_pad;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned ring of stages, then barriers
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + NSTAGE * STAGE_BYTES);
    uint64_t *empty = full + NSTAGE;
    uint64_t *done = empty + NSTAGE;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    int *status = (int *)(tmem_slot + 1); // the producer's status, read by the epilogue

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mt = blockIdx.y, nt = blockIdx.x;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < NSTAGE; ++s)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *status = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    bool ok = true;
    if (threadIdx.x == 0)
    {
        const float *srcs[4];
        // local chunk kc of this segment = global chunk kb + kc
        auto issue = [&](int64_t kc, int s) {
            srcs[0] = a_hi + (mt * kchunks + kb + kc) * (BLOCK_BYTES / 4);
            srcs[1] = a_lo + (mt * kchunks + kb + kc) * (BLOCK_BYTES / 4);
            srcs[2] = b_hi + (nt * kchunks + kb + kc) * (BLOCK_BYTES / 4);
            srcs[3] = b_lo + (nt * kchunks + kb + kc) * (BLOCK_BYTES / 4);
            mbar_expect_tx(&full[s], STAGE_BYTES);
            for (int q = 0; q < 4; ++q)
                bulk_copy_g2s(smem + s * STAGE_BYTES + q * BLOCK_BYTES, srcs[q], BLOCK_BYTES, &full[s]);
        };
        uint32_t full_phase[NSTAGE] = {0, 0}, empty_phase[NSTAGE] = {0, 0};
        int64_t issued = 0;
        for (; issued < nk && issued < NSTAGE; ++issued)
            issue(issued, (int)issued);
        for (int64_t kc = 0; kc < nk && ok; ++kc)
        {
            const int s = (int)(kc % NSTAGE);
            if (!mbar_wait(&full[s], full_phase[s]))
            {
                ok = false;
                break;
            }
            full_phase[s] ^= 1u;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t base = smem_u32(smem + s * STAGE_BYTES);
            for (int ks = 0; ks < TK / 8; ++ks)
            {
                // one k step = 8 tf32 = two 16-byte core-matrix columns
                const uint32_t koff = (uint32_t)ks * 256u;
                const uint64_t dah = smem_desc(base + 0 * BLOCK_BYTES + koff, 128, 1024);
                const uint64_t dal = smem_desc(base + 1 * BLOCK_BYTES + koff, 128, 1024);
                const uint64_t dbh = smem_desc(base + 2 * BLOCK_BYTES + koff, 128, 1024);
                const uint64_t dbl = smem_desc(base + 3 * BLOCK_BYTES + koff, 128, 1024);
                const uint32_t acc0 = (kc > 0 || ks > 0) ? 1u : 0u;
                mma_tf32(tmem, dah, dbh, acc0);
                mma_tf32(tmem, dah, dbl, 1u);
                mma_tf32(tmem, dal, dbh, 1u);
            }
            mma_commit(&empty[s]);
            if (issued < nk)
            {
                // stage s is refilled once the MMAs that read it have completed
                if (!mbar_wait(&empty[s], empty_phase[s]))
                {
                    ok = false;
                    break;
                }
                empty_phase[s] ^= 1u;
                issue(issued, s);
                ++issued;
            }
        }
        // all MMAs issued so far complete before `done` arrives
        mma_commit(done);
        if (!ok)
        {
            atomicExch(&g_tc_error, 1);
            // drain our own copies still in flight (bounded)
            for (int s = 0; s < NSTAGE; ++s)
                (void)mbar_wait(&full[s], full_phase[s]);
        }
        *status = ok ? 1 : 0;
    }
    __syncthreads();
    ok = *status != 0;
    const bool done_ok = mbar_wait(done, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (done_ok && ok)
    {
        // epilogue: warp w reads TMEM lanes 32w..32w+31 = tile rows, 32 columns per load
        const int64_t row = mt * TM + warp * 32 + lane;
        for (int c0 = 0; c0 < TN; c0 += 32)
        {
            uint32_t r[32];
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                         "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                         "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                         : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
                           "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
                           "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
                           "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
                           "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                         : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float *dst = C + row * cols_pad + nt * TN + c0;
#pragma unroll
            for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4 *>(dst + j) = make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]),
                                                                   __uint_as_float(r[j + 2]),
                                                                   __uint_as_float(r[j + 3]));
        }
    }
    else if (threadIdx.x == 0)
    {
        atomicExch(&g_tc_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS)
                     : "memory");
}

// -------------------------------------------------------------- epilogues
// start + the segments' values at idx, in segment order, as an unevaluated
// float pair h + l: Knuth's TwoSum (D. E. Knuth, TAOCP vol. 2, 4.2.2) puts
// each addition's rounding error into l.  In float64 these sums ran on the
// float64 pipe (1/64 of the float32 rate): the n=18 mixed workload's finish
// (1000 x 512 outputs, 45 segments) took 0.19 ms, twice its GEMM.
__device__ __forceinline__ float seg_sum(const float *__restrict__ C, int64_t nseg, int64_t seg_stride, int64_t idx,
                                         float start)
{
    float h = start, l = 0.f;
    const float *c = C + idx;
    for (int64_t z = 0; z < nseg; ++z, c += seg_stride)
    {
        const float x = *c;
        const float s = __fadd_rn(h, x);
        const float bb = __fsub_rn(s, h);
        l = __fadd_rn(l, __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(x, bb)));
        h = s;
    }
    return __fadd_rn(h, l);
}

// expectation: out[k][t] += (C[k][t], C[K+k][t])   (complex64 out)
__global__ void k_finish_expect(const float *__restrict__ C, int64_t nseg, int64_t seg_stride, int64_t cols_pad,
                                int64_t K, int64_t S, float2 *__restrict__ out)
{
    const int64_t total = K * S;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t k = e / S, t = e - k * S;
        float2 o = out[e];
        o.x = seg_sum(C, nseg, seg_stride, k * cols_pad + t, o.x);
        o.y = seg_sum(C, nseg, seg_stride, (K + k) * cols_pad + t, o.y);
        out[e] = o;
    }
}

// weighted: W[p][t] = (C[p][t], C[P+p][t])
__global__ void k_finish_weighted(const float *__restrict__ C, int64_t nseg, int64_t seg_stride, int64_t cols_pad,
                                  int64_t P, int64_t S, float2 *__restrict__ W)
{
    const int64_t total = P * S;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t p = e / S, t = e - p * S;
        W[e] = make_float2(seg_sum(C, nseg, seg_stride, p * cols_pad + t, 0.f),
                           seg_sum(C, nseg, seg_stride, (P + p) * cols_pad + t, 0.f));
    }
}

int64_t round_up(int64_t v, int64_t m)
{
    return (v + m - 1) / m * m;
}

unsigned grid_for(int64_t n)
{
    int64_t b = (n + 255) / 256;
    const int64_t cap = (int64_t)sm_count() * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// 32-deep chunks per float32 accumulation segment: one chunk (12 MMAs of
// K=8) per segment keeps the tensor core's float32 accumulation short.
constexpr int64_t SEG_CHUNKS = 1;

struct GemmLayout
{
    int64_t Mp, Np, Kp, kchunks, nseg;
    float *a_hi, *a_lo, *b_hi, *b_lo, *C;
};

GemmLayout layout(int64_t M, int64_t N, int64_t Kd, void *ws)
{
    GemmLayout g{};
    g.Mp = round_up(M, TM);
    g.Np = round_up(N, TN);
    g.Kp = round_up(Kd, TK);
    g.kchunks = g.Kp / TK;
    g.nseg = (g.kchunks + SEG_CHUNKS - 1) / SEG_CHUNKS;
    float *p = (float *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
    g.a_hi = p;
    g.a_lo = g.a_hi + g.Mp * g.Kp;
    g.b_hi = g.a_lo + g.Mp * g.Kp;
    g.b_lo = g.b_hi + g.Np * g.Kp;
    g.C = g.b_lo + g.Np * g.Kp;
    return g;
}

cudaError_t run_gemm(const GemmLayout &g, cudaStream_t st)
{
    cudaError_t e;
    if ((e = cudaFuncSetAttribute(k_gemm_tf32x3, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES)))
        return e;
    dim3 grid((unsigned)(g.Np / TN), (unsigned)(g.Mp / TM), (unsigned)g.nseg);
    k_gemm_tf32x3<<<grid, 128, SMEM_BYTES, st>>>(g.a_hi, g.a_lo, g.b_hi, g.b_lo, g.kchunks, SEG_CHUNKS, g.Mp, g.Np,
                                                 g.C);
    return launched();
}

} // namespace

size_t tc_workspace_bytes(int64_t M, int64_t N, int64_t Kd)
{
    const GemmLayout g = layout(M, N, Kd, nullptr);
    return (size_t)(2 * g.Mp * g.Kp + 2 * g.Np * g.Kp + g.nseg * g.Mp * g.Np) * sizeof(float) + 256;
}

cudaError_t launch_contract_tc_expect(const void *H, const double *E, int64_t P, int64_t K, int64_t S, void *out,
                                      void *ws, cudaStream_t st)
{
    if (K <= 0 || S <= 0 || P <= 0)
        return cudaSuccess;
    const GemmLayout g = layout(2 * K, S, P, ws);
    cudaError_t e;
    k_prep_a_expect<<<grid_for(g.Mp * g.Kp), 256, 0, st>>>((const float2 *)H, P, K, g.Mp, g.Kp, g.a_hi, g.a_lo);
    if ((e = launched()))
        return e;
    k_prep_b_expect<<<grid_for(g.Np * g.Kp), 256, 0, st>>>(E, P, S, g.Np, g.Kp, g.b_hi, g.b_lo);
    if ((e = launched()))
        return e;
    if ((e = run_gemm(g, st)))
        return e;
    k_finish_expect<<<grid_for(K * S), 256, 0, st>>>(g.C, g.nseg, g.Mp * g.Np, g.Np, K, S, (float2 *)out);
    return launched();
}

cudaError_t launch_weighted_tc(const void *H, const float *X, int64_t P, int64_t K, int64_t S, void *W, void *ws,
                               cudaStream_t st)
{
    if (P <= 0 || S <= 0)
        return cudaSuccess;
    const GemmLayout g = layout(2 * P, S, K, ws);
    cudaError_t e;
    k_prep_a_weighted<<<grid_for(g.Mp * g.Kp), 256, 0, st>>>((const float2 *)H, P, K, g.Mp, g.Kp, g.a_hi, g.a_lo);
    if ((e = launched()))
        return e;
    k_prep_b_weighted<<<grid_for(g.Np * g.Kp), 256, 0, st>>>(X, K, S, g.Np, g.Kp, g.b_hi, g.b_lo);
    if ((e = launched()))
        return e;
    if ((e = run_gemm(g, st)))
        return e;
    k_finish_weighted<<<grid_for(P * S), 256, 0, st>>>(g.C, g.nseg, g.Mp * g.Np, g.Np, P, S, (float2 *)W);
    return launched();
}

// ============================================================================
// Float64 contraction on the tensor cores: digit slices with exact float32
// accumulation (the Ozaki scheme).
//
// Published method: K. Ozaki, T. Ogita, S. Oishi, S. M. Rump, "Error-free
// transformations of matrix multiplication by using fast routines of matrix
// multiplication and its applications", Numer. Algorithms 59 (2012): split
// both operands into slices whose pairwise products are computed without
// rounding by a low-precision matrix engine, then add the slice products in
// high precision.
//
// Here C(M,N) = A(M,Kd) B(N,Kd)^T with A = [Re H^T; Im H^T] (2K x P) and
// B = E^T (S x P), the float64 contraction of SummedPauliOp::
// expectation_value (fast_pauli/cpp/include/__summed_pauli_op.hpp:579-591).
//  * Row scales: row r of A (and of B) gets 2^e_r > max_k |row r|; its element
//    v becomes the integer V = rint(v 2^(55 - e_r)), |V| <= 2^55, an error of
//    at most 2^-56 of the row maximum.
//  * Digits: V = sum_{s=1..8} d_s 128^(8-s) with d_2..d_8 in [-64, 63] and
//    |d_1| <= 65 -- every digit is exact in bf16, every digit product is an
//    integer below 65^2 < 2^12.1.
//  * Levels: the pairs (s, r) with s + r = L have equal weight 128^(16-L) and
//    share a float32 accumulator in TMEM; levels 2..9 are kept (36 of the 64
//    pairs; a term of the first dropped level is below 2^-55 of
//    rowmax * colmax).  A level holds at most 8 pairs, so over a 448-deep k
//    segment its sum stays below 8 * 448 * 65^2 < 2^24 and is exact: the
//    tensor core's float32 accumulation rounds nothing.
//  * Epilogue: per segment, the eight exact level sums of an output are
//    folded into a double-float value (TwoSum); the finishing kernel sums the
//    segments in float64 and applies 2^(e_row + e_col - 12).
// Modelled in numpy on data shaped like the n=14 weight<=2 workload (P = 861,
// Gaussian H, expectation columns with 30x outliers): 1.4e-15 normwise
// against the float64 GEMM (seven digits and levels up to 8: 1.6e-13).  A non-finite value
// in H or E raises the call's flag instead; the float64 CUDA-core GEMM then
// computes the contraction (every kernel here returns at once).
namespace
{

constexpr int OZ_SLICES = 8;                  // digits per element
constexpr int OZ_LMAX = 9;                    // levels 2..OZ_LMAX kept
constexpr int OZ_LEVELS = OZ_LMAX - 1;
constexpr int OZ_TM = 128, OZ_TN = 64, OZ_TK = 16;       // CTA tile, k chunk (bf16 elements)
constexpr int OZ_SBO = 8 * OZ_TK * 2;                    // bytes between 8-row core-matrix groups
constexpr int OZ_A_BLOCK = OZ_TM * OZ_TK * 2;            // 4 KiB
constexpr int OZ_B_BLOCK = OZ_TN * OZ_TK * 2;            // 2 KiB
constexpr int OZ_STAGE = OZ_SLICES * (OZ_A_BLOCK + OZ_B_BLOCK);
constexpr int OZ_NSTAGE = 4;
constexpr int OZ_SMEM = OZ_NSTAGE * OZ_STAGE + 2048; // + 1024-byte alignment pad, barriers
constexpr uint32_t OZ_TMEM_COLS = 512;                   // OZ_LEVELS x OZ_TN
constexpr int64_t OZ_SEG_CHUNKS = 448 / OZ_TK;           // 448-deep exact segments
static_assert((OZ_LMAX - 1) * OZ_SEG_CHUNKS * OZ_TK * 65 * 65 < (1 << 24), "level sums must stay exact");
static_assert(OZ_LEVELS * OZ_TN <= (int)OZ_TMEM_COLS, "levels must fit in TMEM");
static_assert(OZ_SMEM <= 227 * 1024, "stage ring must fit in shared memory");

// kind::f16: D = f32 (bits 4-5 = 1), A = B = bf16 (bits 7-9 and 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
constexpr uint32_t OZ_IDESC =
    (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(OZ_TN >> 3) << 17) | ((uint32_t)(OZ_TM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
                 "l"(da), "l"(db), "r"(OZ_IDESC), "r"(accumulate));
}

// 2^e as a float (-126 <= e <= 127), from its bits
__device__ __forceinline__ float pow2f(int e)
{
    return __uint_as_float((uint32_t)(127 + e) << 23);
}

// byte offset of element (r, k) inside an R x OZ_TK bf16 block
__device__ __forceinline__ uint32_t oz_offset(int r, int k)
{
    return (uint32_t)((r >> 3) * OZ_SBO + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// exponent e with |x| < 2^e for every x of a row whose maximum has these bits
// (0 for an all-zero row, whose digits are all zero)
__device__ __forceinline__ int oz_exponent(unsigned long long maxbits)
{
    const double mx = __longlong_as_double((long long)maxbits);
    int e = 0;
    if (mx > 0.0)
        (void)frexp(mx, &e);
    return e;
}

// Row maxima of A = [Re H^T; Im H^T]: maxbits[m] (m < K: real parts of column
// m of H; K + m: imaginary parts), as bit patterns (non-negative doubles
// order like their bits).  *bad |= a non-finite value.
__global__ void k_oz_max_h(const double2 *__restrict__ H, int64_t P, int64_t K, int64_t rows_per_block,
                           unsigned long long *__restrict__ maxbits, int *__restrict__ bad)
{
    const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K)
        return;
    const int64_t p0 = (int64_t)blockIdx.y * rows_per_block, p1 = min(P, p0 + rows_per_block);
    double mr = 0.0, mi = 0.0;
    bool nf = false;
    for (int64_t p = p0; p < p1; ++p)
    {
        const double2 h = H[p * K + k];
        nf |= !isfinite(h.x) || !isfinite(h.y);
        mr = fmax(mr, fabs(h.x));
        mi = fmax(mi, fabs(h.y));
    }
    if (nf)
        atomicOr(bad, 1);
    atomicMax(&maxbits[k], (unsigned long long)__double_as_longlong(mr));
    atomicMax(&maxbits[K + k], (unsigned long long)__double_as_longlong(mi));
}

// Row maxima of B = E^T: maxbits[t] = max_p |E[p][t]|.
__global__ void k_oz_max_e(const double *__restrict__ E, int64_t P, int64_t S, int64_t rows_per_block,
                           unsigned long long *__restrict__ maxbits, int *__restrict__ bad)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= S)
        return;
    const int64_t p0 = (int64_t)blockIdx.y * rows_per_block, p1 = min(P, p0 + rows_per_block);
    double m = 0.0;
    bool nf = false;
    for (int64_t p = p0; p < p1; ++p)
    {
        const double v = E[p * S + t];
        nf |= !isfinite(v);
        m = fmax(m, fabs(v));
    }
    if (nf)
        atomicOr(bad, 1);
    atomicMax(&maxbits[t], (unsigned long long)__double_as_longlong(m));
}

// The seven digit slices of an operand, each in OZ_TK-deep blocks of
// tile_rows rows in the canonical K-major core-matrix layout:
// block (s, row tile, k chunk) at ((s * tiles + tile) * kchunks + chunk).
// One thread per (row, 8-deep k group) writes 16 bytes per slice.
// A operand (IS_H): element (m, p) = m < K ? Re H[p][m] : Im H[p][m-K];
// B operand: element (t, p) = E[p][t].
template <bool IS_H>
__global__ void k_oz_slice(const void *__restrict__ src, int64_t P, int64_t width, int64_t rows, int64_t rows_pad,
                           int64_t depth_pad, int tile_rows, const unsigned long long *__restrict__ maxbits,
                           const int *__restrict__ skip_if, unsigned char *__restrict__ slices, int *__restrict__ exps)
{
    if (*skip_if)
        return;
    const int64_t kgroups = depth_pad / 8, kchunks = depth_pad / OZ_TK, tiles = rows_pad / tile_rows;
    const int64_t block_bytes = (int64_t)tile_rows * OZ_TK * 2;
    const int64_t total = rows_pad * kgroups;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t r = e % rows_pad, kg = e / rows_pad;
        const int ex = r < rows ? oz_exponent(maxbits[r]) : 0;
        if (kg == 0)
            exps[r] = ex;
        uint32_t packed[OZ_SLICES][4];
#pragma unroll
        for (int j = 0; j < 8; ++j)
        {
            const int64_t k = kg * 8 + j;
            double v = 0.0;
            if (r < rows && k < P)
            {
                if constexpr (IS_H)
                {
                    const double2 *H = (const double2 *)src;
                    v = r < width ? H[k * width + r].x : H[k * width + (r - width)].y;
                }
                else
                {
                    v = ((const double *)src)[k * width + r];
                }
            }
            long long n = llrint(ldexp(v, 55 - ex)); // |n| <= 2^55
            int d[OZ_SLICES];
#pragma unroll
            for (int s = OZ_SLICES - 1; s >= 1; --s)
            {
                d[s] = (int)((n + 64) & 127) - 64; // balanced digit in [-64, 63]
                n = (n - d[s]) >> 7;               // exact: n - d[s] is a multiple of 128
            }
            d[0] = (int)n; // |d_1| <= 2^55 / 128^7 + 1/2 -> <= 65
#pragma unroll
            for (int s = 0; s < OZ_SLICES; ++s)
            {
                // an integer of magnitude <= 256 is exact in bf16: its bits are
                // the top half of the float's
                const uint32_t b = __float_as_uint((float)d[s]) >> 16;
                if (j & 1)
                    packed[s][j >> 1] |= b << 16;
                else
                    packed[s][j >> 1] = b;
            }
        }
        const int64_t tile = r / tile_rows, chunk = kg / (OZ_TK / 8);
        const uint32_t off = oz_offset((int)(r % tile_rows), (int)(kg % (OZ_TK / 8)) * 8);
#pragma unroll
        for (int s = 0; s < OZ_SLICES; ++s)
        {
            unsigned char *dst = slices + ((s * tiles + tile) * kchunks + chunk) * block_bytes + off;
            *reinterpret_cast<uint4 *>(dst) = make_uint4(packed[s][0], packed[s][1], packed[s][2], packed[s][3]);
        }
    }
}

// One 128 x 64 tile of one k segment (seg_chunks <= OZ_SEG_CHUNKS k chunks,
// at most 448 deep) per CTA (blockIdx.z = segment): the level sums
// accumulate in TMEM (level L at columns (L-2) * 64), and the epilogue writes
// each output's folded double-float value (hi, lo) of the segment to C[z]
// (rows_pad x cols_pad float2).
__global__ void __launch_bounds__(128, 1)
    k_gemm_oz(const unsigned char *__restrict__ a_sl, const unsigned char *__restrict__ b_sl, int64_t kchunks,
              int64_t seg_chunks, int64_t mtiles, int64_t ntiles, int64_t rows_pad, int64_t cols_pad,
              float2 *__restrict__ C, const int *__restrict__ skip_if)
{
    if (*skip_if)
        return;
    const int64_t kb = (int64_t)blockIdx.z * seg_chunks;
    const int64_t nk = min(kchunks, kb + seg_chunks) - kb; // chunks of this segment (>= 1)
    C += (int64_t)blockIdx.z * rows_pad * cols_pad;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *full = (uint64_t *)(smem + OZ_NSTAGE * OZ_STAGE);
    uint64_t *empty = full + OZ_NSTAGE;
    uint64_t *done = empty + OZ_NSTAGE;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    int *status = (int *)(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t mt = blockIdx.y, nt = blockIdx.x;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < OZ_NSTAGE; ++s)
        {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        *status = 1;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tmem_slot)),
                     "r"(OZ_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = *tmem_slot;

    if (threadIdx.x == 0)
    {
        bool ok = true;
        auto issue = [&](int64_t kc, int s) {
            unsigned char *stage = smem + s * OZ_STAGE;
            mbar_expect_tx(&full[s], OZ_STAGE);
            for (int q = 0; q < OZ_SLICES; ++q)
                bulk_copy_g2s(stage + q * OZ_A_BLOCK, a_sl + ((q * mtiles + mt) * kchunks + kb + kc) * OZ_A_BLOCK,
                              OZ_A_BLOCK, &full[s]);
            for (int q = 0; q < OZ_SLICES; ++q)
                bulk_copy_g2s(stage + OZ_SLICES * OZ_A_BLOCK + q * OZ_B_BLOCK,
                              b_sl + ((q * ntiles + nt) * kchunks + kb + kc) * OZ_B_BLOCK, OZ_B_BLOCK, &full[s]);
        };
        uint32_t full_phase[OZ_NSTAGE], empty_phase[OZ_NSTAGE];
        bool pending[OZ_NSTAGE];
        for (int s = 0; s < OZ_NSTAGE; ++s)
        {
            full_phase[s] = empty_phase[s] = 0;
            pending[s] = false;
        }
        int64_t issued = 0;
        for (; issued < nk && issued < OZ_NSTAGE; ++issued)
        {
            issue(issued, (int)issued);
            pending[issued] = true;
        }
        for (int64_t kc = 0; kc < nk; ++kc)
        {
            const int s = (int)(kc % OZ_NSTAGE);
            if (!mbar_wait(&full[s], full_phase[s]))
            {
                ok = false;
                break;
            }
            full_phase[s] ^= 1u;
            pending[s] = false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // the descriptor's start field is address >> 4 in its low 14 bits
            // (shared addresses < 256 KiB), so the descriptor of a block at
            // byte offset o from the stage is the stage's descriptor + o / 16:
            // one add per MMA, the rest folds into constants
            const uint64_t d0 = smem_desc(smem_u32(smem + s * OZ_STAGE), 128, OZ_SBO);
            const uint32_t first = kc > 0 ? 1u : 0u;
#pragma unroll
            for (int L = 2; L <= OZ_LMAX; ++L)
            {
                constexpr int kA = OZ_A_BLOCK / 16, kB = OZ_B_BLOCK / 16, kB0 = OZ_SLICES * OZ_A_BLOCK / 16;
                const int s_lo = L - OZ_SLICES > 1 ? L - OZ_SLICES : 1;
                const int s_hi = L - 1 < OZ_SLICES ? L - 1 : OZ_SLICES;
#pragma unroll
                for (int sa = s_lo; sa <= s_hi; ++sa)
                {
                    const int sb = L - sa;
                    const uint64_t da = d0 + (uint64_t)((sa - 1) * kA);
                    const uint64_t db = d0 + (uint64_t)(kB0 + (sb - 1) * kB);
                    mma_bf16(tmem + (uint32_t)((L - 2) * OZ_TN), da, db, sa > s_lo ? 1u : first);
                }
            }
            mma_commit(&empty[s]);
            // refill the stage of the previous chunk, whose MMAs were issued
            // one chunk earlier (one chunk of MMAs stays queued meanwhile)
            if (kc >= 1 && issued < nk)
            {
                const int sp = (int)((kc - 1) % OZ_NSTAGE);
                if (!mbar_wait(&empty[sp], empty_phase[sp]))
                {
                    ok = false;
                    break;
                }
                empty_phase[sp] ^= 1u;
                issue(issued, sp);
                pending[sp] = true;
                ++issued;
            }
        }
        mma_commit(done);
        if (!ok)
        {
            atomicExch(&g_tc_error, 1);
            // drain our own copies still in flight (bounded)
            for (int s = 0; s < OZ_NSTAGE; ++s)
                if (pending[s])
                    (void)mbar_wait(&full[s], full_phase[s]);
        }
        *status = ok ? 1 : 0;
    }
    __syncthreads();
    const bool ok = *status != 0;
    const bool done_ok = mbar_wait(done, 0);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

    if (done_ok && ok)
    {
        const int64_t row = mt * OZ_TM + warp * 32 + lane;
        float2 *dst_row = C + row * cols_pad + nt * OZ_TN;
        for (int c0 = 0; c0 < OZ_TN; c0 += 8)
        {
            uint32_t v[OZ_LEVELS][8];
#pragma unroll
            for (int l = 0; l < OZ_LEVELS; ++l)
            {
                const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(l * OZ_TN + c0);
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                             : "=r"(v[l][0]), "=r"(v[l][1]), "=r"(v[l][2]), "=r"(v[l][3]), "=r"(v[l][4]),
                               "=r"(v[l][5]), "=r"(v[l][6]), "=r"(v[l][7])
                             : "r"(taddr));
            }
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float2 out[8];
#pragma unroll
            for (int j = 0; j < 8; ++j)
            {
                // level L (index l = L - 2) weighs 128^(-l) relative to level 2;
                // add from the smallest weight up, exactly (TwoSum)
                float hi = __fmul_rn(__uint_as_float(v[OZ_LEVELS - 1][j]), pow2f(-7 * (OZ_LEVELS - 1)));
                float lo = 0.0f;
#pragma unroll
                for (int l = OZ_LEVELS - 2; l >= 0; --l)
                {
                    const float t = __fmul_rn(__uint_as_float(v[l][j]), pow2f(-7 * l));
                    const float s = __fadd_rn(hi, t);
                    const float bb = __fsub_rn(s, hi);
                    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(t, bb));
                    hi = s;
                    lo = __fadd_rn(lo, err);
                }
                const float s = __fadd_rn(hi, lo);
                out[j] = make_float2(s, __fsub_rn(lo, __fsub_rn(s, hi)));
            }
#pragma unroll
            for (int j = 0; j < 8; j += 2)
                *reinterpret_cast<float4 *>(dst_row + c0 + j) = make_float4(out[j].x, out[j].y, out[j + 1].x,
                                                                            out[j + 1].y);
        }
    }
    else if (threadIdx.x == 0)
    {
        atomicExch(&g_tc_error, 1);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(OZ_TMEM_COLS)
                     : "memory");
}

// (h, l) += (bh, bl) in double-float (TwoSum, then the low parts)
__device__ __forceinline__ void oz_df_add(float &h, float &l, float bh, float bl)
{
    const float s = __fadd_rn(h, bh);
    const float bb = __fsub_rn(s, h);
    const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(bh, bb));
    h = s;
    l = __fadd_rn(l, __fadd_rn(err, bl));
}

// v * 2^e, exact: the power of two from its bits when it is a normal double
__device__ __forceinline__ double oz_scale(double v, int e)
{
    if (e >= -1022 && e <= 1023)
        return v * __longlong_as_double((long long)(e + 1023) << 52);
    return ldexp(v, e);
}

// out[k][t] += (sum_z C[z][k][t], sum_z C[z][K+k][t]) * 2^(e_row + e_col - 12);
// segments summed in double-float, float64 only for the scale and the add
__global__ void k_oz_finish(const float2 *__restrict__ C, int64_t nseg, int64_t seg_stride, int64_t cols_pad,
                            int64_t K, int64_t S, const int *__restrict__ exp_a, const int *__restrict__ exp_b,
                            const int *__restrict__ skip_if, double2 *__restrict__ out)
{
    if (*skip_if)
        return;
    const int64_t total = K * S;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t k = e / S, t = e - k * S;
        const float2 *ca = C + k * cols_pad + t, *cb = C + (K + k) * cols_pad + t;
        float2 a = ca[0], b = cb[0];
        for (int64_t z = 1; z < nseg; ++z)
        {
            const float2 a2 = ca[z * seg_stride], b2 = cb[z * seg_stride];
            oz_df_add(a.x, a.y, a2.x, a2.y);
            oz_df_add(b.x, b.y, b2.x, b2.y);
        }
        const int eb = exp_b[t] - 12;
        double2 o = out[e];
        o.x += oz_scale((double)a.x + (double)a.y, exp_a[k] + eb);
        o.y += oz_scale((double)b.x + (double)b.y, exp_a[K + k] + eb);
        out[e] = o;
    }
}

struct OzLayout
{
    int64_t Mp, Np, Kp, kchunks, seg_chunks, nseg;
    unsigned long long *max_a, *max_b;
    int *exp_a, *exp_b;
    unsigned char *a_sl, *b_sl;
    float2 *C;
};

OzLayout oz_layout(int64_t M, int64_t N, int64_t Kd, void *ws)
{
    OzLayout g{};
    g.Mp = round_up(M, OZ_TM);
    g.Np = round_up(N, OZ_TN);
    g.Kp = round_up(Kd, OZ_TK);
    g.kchunks = g.Kp / OZ_TK;
    // segments of at most OZ_SEG_CHUNKS k chunks (their level sums stay
    // exact); more, shorter ones while the output tiles alone would leave SMs
    // idle (one CTA per SM: each holds all of TMEM), up to one CTA per SM --
    // a narrow call's GEMM then takes a fraction of one long segment's time
    const int64_t tiles = (g.Mp / OZ_TM) * (g.Np / OZ_TN);
    int64_t nseg = (g.kchunks + OZ_SEG_CHUNKS - 1) / OZ_SEG_CHUNKS;
    nseg = std::max<int64_t>(nseg, std::min<int64_t>(g.kchunks, (int64_t)sm_count() / std::max<int64_t>(1, tiles)));
    g.seg_chunks = (g.kchunks + nseg - 1) / nseg;
    g.nseg = (g.kchunks + g.seg_chunks - 1) / g.seg_chunks;
    unsigned char *p = (unsigned char *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
    g.max_a = (unsigned long long *)p;
    g.max_b = g.max_a + g.Mp;
    p += round_up((g.Mp + g.Np) * 8, 256);
    g.exp_a = (int *)p;
    g.exp_b = g.exp_a + g.Mp;
    p += round_up((g.Mp + g.Np) * 4, 256);
    g.a_sl = p;
    p += OZ_SLICES * g.Mp * g.Kp * 2;
    g.b_sl = p;
    p += OZ_SLICES * g.Np * g.Kp * 2;
    g.C = (float2 *)p;
    return g;
}

} // namespace

size_t oz_workspace_bytes(int64_t M, int64_t N, int64_t Kd)
{
    const OzLayout g = oz_layout(M, N, Kd, nullptr);
    return (size_t)(round_up((g.Mp + g.Np) * 8, 256) + round_up((g.Mp + g.Np) * 4, 256) +
                    OZ_SLICES * (g.Mp + g.Np) * g.Kp * 2 +
                    g.nseg * g.Mp * g.Np * 8) +
           256;
}

namespace
{
int64_t oz_rows_per_block(int64_t P)
{
    return P > 8 * 4096 ? (P + 4095) / 4096 : 8; // grid y <= 4096
}
} // namespace

cudaError_t launch_contract_oz_prep_h(const void *H, int64_t P, int64_t K, int64_t S, void *ws, int *flag,
                                      cudaStream_t st)
{
    if (K <= 0 || S <= 0 || P <= 0)
        return cudaSuccess;
    const OzLayout g = oz_layout(2 * K, S, P, ws);
    cudaError_t e;
    if ((e = cudaMemsetAsync(g.max_a, 0, (size_t)g.Mp * 8, st)))
        return e;
    const int64_t rows_per_block = oz_rows_per_block(P);
    const unsigned py = (unsigned)((P + rows_per_block - 1) / rows_per_block);
    k_oz_max_h<<<dim3((unsigned)((K + 127) / 128), py), 128, 0, st>>>((const double2 *)H, P, K, rows_per_block,
                                                                      g.max_a, flag);
    if ((e = launched()))
        return e;
    k_oz_slice<true><<<grid_for(g.Mp * (g.Kp / 8)), 256, 0, st>>>(H, P, K, 2 * K, g.Mp, g.Kp, OZ_TM, g.max_a, flag,
                                                                  g.a_sl, g.exp_a);
    return launched();
}

cudaError_t launch_contract_oz_expect(const void *H, const double *E, int64_t P, int64_t K, int64_t S, void *out,
                                      void *ws, int *flag, cudaStream_t st)
{
    if (K <= 0 || S <= 0 || P <= 0)
        return cudaSuccess;
    const OzLayout g = oz_layout(2 * K, S, P, ws);
    cudaError_t e;
    if ((e = cudaMemsetAsync(g.max_b, 0, (size_t)g.Np * 8, st)))
        return e;
    const int64_t rows_per_block = oz_rows_per_block(P);
    const unsigned py = (unsigned)((P + rows_per_block - 1) / rows_per_block);
    k_oz_max_e<<<dim3((unsigned)((S + 127) / 128), py), 128, 0, st>>>(E, P, S, rows_per_block, g.max_b, flag);
    if ((e = launched()))
        return e;
    k_oz_slice<false><<<grid_for(g.Np * (g.Kp / 8)), 256, 0, st>>>(E, P, S, S, g.Np, g.Kp, OZ_TN, g.max_b, flag,
                                                                   g.b_sl, g.exp_b);
    if ((e = launched()))
        return e;
    if ((e = cudaFuncSetAttribute(k_gemm_oz, cudaFuncAttributeMaxDynamicSharedMemorySize, OZ_SMEM)))
        return e;
    dim3 grid((unsigned)(g.Np / OZ_TN), (unsigned)(g.Mp / OZ_TM), (unsigned)g.nseg);
    k_gemm_oz<<<grid, 128, OZ_SMEM, st>>>(g.a_sl, g.b_sl, g.kchunks, g.seg_chunks, g.Mp / OZ_TM, g.Np / OZ_TN, g.Mp,
                                          g.Np, g.C, flag);
    if ((e = launched()))
        return e;
    k_oz_finish<<<grid_for(K * S), 256, 0, st>>>(g.C, g.nseg, g.Mp * g.Np, g.Np, K, S, g.exp_a, g.exp_b, flag,
                                                 (double2 *)out);
    return launched();
}

cudaError_t read_device_error(int *code, cudaStream_t st)
{
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(&v, g_tc_error, sizeof(int), 0, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
    *code = v;
    const int zero = 0;
    return cudaMemcpyToSymbolAsync(g_tc_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, st);
}

} // namespace fpg
