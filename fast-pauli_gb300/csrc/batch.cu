// batch.cu -- many expectation problems of uneven size in one persistent,
// graph-capturable launch sequence, with a project-written autotuner.
//
// A batch holds problems (operator, coefficients (P,K), states (2^n,S),
// output (K,S)) of different qubit counts, string counts and state counts --
// e.g. 256 PauliOp.expectation_value calls (reference __pauli_op.hpp:482-549)
// that would otherwise be 256 separate calls.  Planning turns every problem
// into work items (entry, chunk, column tile, row split) of the expectation
// kernel; one persistent kernel per (chunk class, vector width) bucket pulls
// items from a device work queue (atomic counter), so small problems fill the
// gaps left by large ones and no launch is wasted on a tail (tuning
// ctas_per_sm = -1 instead launches one CTA per item and lets the hardware
// block scheduler drain them; the autotuner picks).  Item
// order: problems largest first, then column tile, row split, chunk (chunks
// fastest, so concurrently running CTAs share rows in L2).  Partial sums go
// to per-problem (split, string, state) tables, reduced in place in a fixed
// order, then one batched kernel contracts them with the coefficients in
// float64 and OVERWRITES the outputs.  Every summation order is fixed, so a
// problem's result does not depend on what else is in the batch or on how
// the work queue was drained.
//
// fpg_batch_run enqueues: counter reset (memset), the persistent kernels, the
// reduction and the contraction -- no allocation, so the sequence can be
// captured into a CUDA graph (fpg_batch_run_graph captures once and replays).
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "fpg.h"

#include "expect_body.cuh"
#include "host_internal.hpp"

namespace fpg
{

struct BatchEntry
{
    const void *psi;
    double *partial; // (n_splits, P, S)
    const StringRec *recs;
    const int32_t *orig;
    const Chunk *chunks;
    const void *coeffs; // (P, K) complex
    void *out;          // (K, S) complex
    int64_t S;
    int64_t P;
    int64_t K;
    int64_t red_off; // offset in the flattened (P*S) index space of the reduction
    int64_t con_off; // offset in the flattened (K*S) index space of the contraction
    int32_t n;
    int32_t TC;
    int32_t n_splits;
    int32_t V; // complex elements per lane (2 only for complex64 with an even state count)
};

constexpr int kBuckets = 2 * kNumChunkClasses; // (chunk class, V in {1, 2})

struct BatchItem
{
    int32_t entry;
    int32_t chunk;
    int32_t ctile;
    int32_t split;
};

namespace
{

// float32 chunks of up to four strings do little arithmetic per row and are
// bound by memory latency: ask the compiler for three resident 256-thread CTAs
// per SM (<= 85 registers), as the per-call kernel does.  Larger chunks and
// float64 keep the default.
template <typename T, int G> constexpr int kBatchMinBlocks = (sizeof(T) == 4 && G <= 4) ? 3 : 1;

template <typename T, int V, int GE, int GO>
__global__ void __launch_bounds__(256, kBatchMinBlocks<T, GE + GO>) k_batch_expect(const BatchEntry *__restrict__ entries,
                                                      const BatchItem *__restrict__ items, int n_items,
                                                      int *__restrict__ counter)
{
    extern __shared__ double red[]; // blockDim.x * V doubles
    __shared__ int s_item;
    for (;;)
    {
        if (threadIdx.x == 0)
            s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_item;
        __syncthreads();
        if (it >= n_items)
            break;
        const BatchItem bi = items[it];
        const BatchEntry &e = entries[bi.entry];
        expect_chunk_body<T, V, GE, GO>((const T *)e.psi, e.S, e.n, e.recs, e.orig, e.P, e.chunks[bi.chunk], e.TC,
                                        (int64_t)bi.ctile, bi.split, e.n_splits, e.partial, red);
    }
}

// Item-grid form: one CTA per work item (blockIdx.x); the hardware block
// scheduler hands out items as SMs free up.  Same work as the persistent form
// without its loop-carried state.
template <typename T, int V, int GE, int GO>
__global__ void __launch_bounds__(256, kBatchMinBlocks<T, GE + GO>) k_batch_items(const BatchEntry *__restrict__ entries,
                                                     const BatchItem *__restrict__ items)
{
    extern __shared__ double red[]; // blockDim.x * V doubles
    const BatchItem bi = items[blockIdx.x];
    const BatchEntry &e = entries[bi.entry];
    expect_chunk_body<T, V, GE, GO>((const T *)e.psi, e.S, e.n, e.recs, e.orig, e.P, e.chunks[bi.chunk], e.TC,
                                    (int64_t)bi.ctile, bi.split, e.n_splits, e.partial, red);
}

__device__ __forceinline__ int find_entry(const BatchEntry *entries, int n_entries, int64_t idx, bool contraction)
{
    int lo = 0, hi = n_entries - 1;
    while (lo < hi)
    {
        const int mid = (lo + hi + 1) >> 1;
        const int64_t off = contraction ? entries[mid].con_off : entries[mid].red_off;
        if (off <= idx)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// partial[0] = sum over splits, per problem, in split order
__global__ void k_batch_reduce(const BatchEntry *__restrict__ entries, int n_entries, int64_t total)
{
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    {
        const BatchEntry &e = entries[find_entry(entries, n_entries, g, false)];
        if (e.n_splits <= 1)
            continue;
        const int64_t i = g - e.red_off, cnt = e.P * e.S;
        double s = e.partial[i];
        for (int p = 1; p < e.n_splits; ++p)
            s += e.partial[(int64_t)p * cnt + i];
        e.partial[i] = s;
    }
}

// out(k,t) = sum_j coeffs(j,k) ev(j,t)
template <typename CT>
__global__ void k_batch_contract(const BatchEntry *__restrict__ entries, int n_entries, int64_t total)
{
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    {
        const BatchEntry &e = entries[find_entry(entries, n_entries, g, true)];
        const int64_t i = g - e.con_off;
        const int64_t k = i / e.S, t = i - k * e.S;
        const CT *h = (const CT *)e.coeffs;
        double re = 0.0, im = 0.0;
        for (int64_t j = 0; j < e.P; ++j)
        {
            const CT c = h[j * e.K + k];
            const double v = e.partial[j * e.S + t];
            re = fma((double)c.x, v, re);
            im = fma((double)c.y, v, im);
        }
        CT o;
        o.x = re;
        o.y = im;
        ((CT *)e.out)[k * e.S + t] = o;
    }
}

} // namespace
} // namespace fpg

using namespace fpg;

struct fpg_batch
{
    int32_t dtype = FPG_C64;
    int device = 0;
    struct Problem
    {
        const fpg_operator *op;
        const void *coeffs;
        int64_t K;
        const void *psi;
        void *out;
        int64_t S;
    };
    std::vector<Problem> problems;
    fpg_batch_tuning tuning{256, 0, 1 << 15, 40};
    bool planned = false;
    // device state of the plan
    BatchEntry *d_entries = nullptr;
    BatchItem *d_items = nullptr;
    int *d_counters = nullptr;
    double *d_partial = nullptr;
    int bucket_begin[kBuckets + 1] = {}; // items of bucket (class, V) contiguous
    int64_t red_total = 0, con_total = 0;
    int grid = 0;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;

    void free_plan()
    {
        if (exec)
            cudaGraphExecDestroy(exec);
        if (graph)
            cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        cudaFree(d_entries);
        cudaFree(d_items);
        cudaFree(d_counters);
        cudaFree(d_partial);
        d_entries = nullptr;
        d_items = nullptr;
        d_counters = nullptr;
        d_partial = nullptr;
        planned = false;
    }
};

namespace
{

int tc_for(int64_t S)
{
    int tc = 1;
    while (tc < 32 && tc < S)
        tc <<= 1;
    return tc;
}

template <typename T, int V>
cudaError_t launch_class_v(int cls, int grid, int threads, const BatchEntry *e, const BatchItem *items, int n_items,
                           int *counter, cudaStream_t st)
{
    const size_t smem = (size_t)threads * V * sizeof(double);
    // grid < 0: item-grid form (one CTA per item)
#define FPG_BCASE(ID, GE, GO)                                                                                          \
    case ID:                                                                                                           \
        if (grid < 0)                                                                                                  \
            k_batch_items<T, V, GE, GO><<<(unsigned)n_items, threads, smem, st>>>(e, items);                           \
        else                                                                                                           \
            k_batch_expect<T, V, GE, GO><<<grid, threads, smem, st>>>(e, items, n_items, counter);                    \
        break;
    switch (cls)
    {
        FPG_BCASE(0, 1, 0)
        FPG_BCASE(1, 0, 1)
        FPG_BCASE(2, 1, 1)
        FPG_BCASE(3, 2, 2)
        FPG_BCASE(4, 4, 4)
        FPG_BCASE(5, 8, 8)
        FPG_BCASE(6, 8, 0)
        FPG_BCASE(7, 0, 8)
    default:
        return cudaErrorInvalidValue;
    }
#undef FPG_BCASE
    return launched();
}

template <typename T, int V> int max_resident_v(int cls, int threads)
{
    int nb = 0;
    const size_t smem = (size_t)threads * V * sizeof(double);
    cudaError_t e = cudaErrorInvalidValue;
#define FPG_OCC(ID, GE, GO)                                                                                            \
    case ID:                                                                                                           \
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch_expect<T, V, GE, GO>, threads, smem);           \
        break;
    switch (cls)
    {
        FPG_OCC(0, 1, 0)
        FPG_OCC(1, 0, 1)
        FPG_OCC(2, 1, 1)
        FPG_OCC(3, 2, 2)
        FPG_OCC(4, 4, 4)
        FPG_OCC(5, 8, 8)
        FPG_OCC(6, 8, 0)
        FPG_OCC(7, 0, 8)
    default:
        break;
    }
#undef FPG_OCC
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return nb < 1 ? 1 : nb;
}

// bucket = 2 * class + (V - 1); V = 2 exists for complex64 only
cudaError_t launch_bucket(bool fp32, int bucket, int grid, int threads, const BatchEntry *e, const BatchItem *items,
                          int n_items, int *counter, cudaStream_t st)
{
    const int cls = bucket / 2, V = bucket % 2 + 1;
    if (!fp32)
        return V == 1 ? launch_class_v<double, 1>(cls, grid, threads, e, items, n_items, counter, st)
                      : cudaErrorInvalidValue;
    return V == 1 ? launch_class_v<float, 1>(cls, grid, threads, e, items, n_items, counter, st)
                  : launch_class_v<float, 2>(cls, grid, threads, e, items, n_items, counter, st);
}

int max_resident(bool fp32, int bucket, int threads)
{
    const int cls = bucket / 2, V = bucket % 2 + 1;
    if (!fp32)
        return max_resident_v<double, 1>(cls, threads);
    return V == 1 ? max_resident_v<float, 1>(cls, threads) : max_resident_v<float, 2>(cls, threads);
}

// Host side of a plan: per-problem entries (tiling, row splits, offsets of
// the flattened reduction and contraction index spaces) and the work items
// bucketed by (chunk class, V), largest problems first.  Device pointers of
// the entries' partial tables are filled in by the caller (partial_off[i] =
// the offset of problem i's table in one buffer of partial_total doubles).
struct HostPlan
{
    std::vector<BatchEntry> entries;
    std::vector<BatchItem> items;
    std::vector<int64_t> partial_off;
    int bucket_begin[kBuckets + 1] = {};
    int64_t red_total = 0, con_total = 0, partial_total = 0;
};

// Tiling of one problem, the rules of a single call: vector width,
// L2-line-wide column tiles, and row windows (splits) only when a column tile
// cannot stay in L2.
void entry_tiling(const fpg_operator *op, int64_t S, const void *psi, bool fp32, const fpg_batch_tuning &t,
                  int32_t &V, int32_t &TC, int32_t &n_splits)
{
    const int64_t tile_budget = (int64_t)t.tile_mb << 20;
    V = (fp32 && S % 2 == 0 && ((uintptr_t)psi % 16) == 0) ? 2 : 1;
    const int bpl = V * (fp32 ? 8 : 16);
    TC = column_lanes_for_l2(std::min(tc_for((S + V - 1) / V), t.threads_per_cta), op->n, bpl, tile_budget);
    const int64_t NB = op->n >= 5 ? ((int64_t)1 << (op->n - 5)) : 1;
    const int64_t window = std::max<int64_t>(1, t.rows_per_item / 32);
    n_splits = 1;
    if (column_tile_footprint(TC, op->n, bpl) > tile_budget)
        n_splits = (int32_t)std::max<int64_t>(1, std::min<int64_t>(256, (NB / 2 + window - 1) / window));
}

int plan_host(const std::vector<fpg_batch::Problem> &problems, bool fp32, const fpg_batch_tuning &t, HostPlan &hp)
{
    const int np = (int)problems.size();
    // largest problems first
    std::vector<int> order((size_t)np);
    for (int i = 0; i < np; ++i)
        order[(size_t)i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) {
        const auto &pa = problems[(size_t)a], &pc = problems[(size_t)c];
        const double wa = (double)pa.op->P * (double)(1ll << pa.op->n) * (double)pa.S;
        const double wc = (double)pc.op->P * (double)(1ll << pc.op->n) * (double)pc.S;
        return wa > wc;
    });
    hp.entries.assign((size_t)np, BatchEntry{});
    std::vector<std::vector<BatchItem>> by_bucket(kBuckets);
    for (int pos = 0; pos < np; ++pos)
    {
        const int i = order[(size_t)pos];
        const auto &p = problems[(size_t)i];
        const fpg_operator *op = p.op;
        BatchEntry &e = hp.entries[(size_t)i];
        e.psi = p.psi;
        e.recs = op->d_recs;
        e.orig = op->d_orig;
        e.chunks = op->d_chunks;
        e.coeffs = p.coeffs;
        e.out = p.out;
        e.S = p.S;
        e.P = op->P;
        e.K = p.K;
        e.n = op->n;
        entry_tiling(op, p.S, p.psi, fp32, t, e.V, e.TC, e.n_splits);
        const int64_t ctiles = (e.S + (int64_t)e.TC * e.V - 1) / ((int64_t)e.TC * e.V);
        for (int c = 0; c < kNumChunkClasses; ++c)
        {
            auto &dst = by_bucket[(size_t)(2 * c + (e.V - 1))];
            for (int64_t ct = 0; ct < ctiles; ++ct)
                for (int s = 0; s < e.n_splits; ++s)
                    for (int ch = op->class_begin[(size_t)c]; ch < op->class_begin[(size_t)c + 1]; ++ch)
                        dst.push_back(BatchItem{i, ch, (int32_t)ct, s});
        }
    }
    hp.items.clear();
    for (int k = 0; k < kBuckets; ++k)
    {
        hp.bucket_begin[k] = (int)hp.items.size();
        hp.items.insert(hp.items.end(), by_bucket[(size_t)k].begin(), by_bucket[(size_t)k].end());
    }
    hp.bucket_begin[kBuckets] = (int)hp.items.size();
    if (hp.items.size() > (size_t)0x7fffffff)
        return set_error(FPG_ERR_UNSUPPORTED, "batch has too many work items");
    // entries keep the order of addition: partial tables and the flattened
    // index spaces of reduction and contraction are laid out in that order
    hp.partial_off.assign((size_t)np, 0);
    int64_t red_off = 0, con_off = 0, partial_total = 0;
    for (int i = 0; i < np; ++i)
    {
        BatchEntry &e = hp.entries[(size_t)i];
        e.red_off = red_off;
        e.con_off = con_off;
        red_off += e.P * e.S;
        con_off += e.K * e.S;
        hp.partial_off[(size_t)i] = partial_total;
        partial_total += (int64_t)e.n_splits * e.P * e.S;
    }
    hp.red_total = red_off;
    hp.con_total = con_off;
    hp.partial_total = partial_total;
    return FPG_OK;
}

int check_tuning(const fpg_batch_tuning &t)
{
    if (t.threads_per_cta != 128 && t.threads_per_cta != 256)
        return set_error(FPG_ERR_INVALID, "threads_per_cta must be 128 or 256");
    if (t.ctas_per_sm < -1 || t.ctas_per_sm > 8)
        return set_error(FPG_ERR_INVALID,
                         "ctas_per_sm must be in [-1, 8] (0: as many as fit; -1: one CTA per work item)");
    if (t.rows_per_item < 32 || (t.rows_per_item & (t.rows_per_item - 1)))
        return set_error(FPG_ERR_INVALID, "rows_per_item must be a power of two >= 32");
    if (t.tile_mb < 1)
        return set_error(FPG_ERR_INVALID, "tile_mb must be >= 1");
    return FPG_OK;
}

int do_plan(fpg_batch *b, const fpg_batch_tuning &t)
{
    if (int rc = check_tuning(t))
        return rc;
    b->free_plan();
    const bool fp32 = b->dtype == FPG_C64;
    HostPlan hp;
    if (int rc = plan_host(b->problems, fp32, t, hp))
        return rc;
    std::copy(hp.bucket_begin, hp.bucket_begin + kBuckets + 1, b->bucket_begin);
    b->red_total = hp.red_total;
    b->con_total = hp.con_total;
    cudaError_t err = cudaSuccess;
    if ((err = cudaMalloc((void **)&b->d_partial, (size_t)std::max<int64_t>(1, hp.partial_total) * sizeof(double))))
    {
        b->free_plan();
        return cuda_error(err, "fpg_batch_plan: partial tables");
    }
    for (size_t i = 0; i < hp.entries.size(); ++i)
        hp.entries[i].partial = b->d_partial + hp.partial_off[i];
    auto &entries = hp.entries;
    auto &items = hp.items;
    if ((err = cudaMalloc((void **)&b->d_entries, entries.size() * sizeof(BatchEntry))) ||
        (err = cudaMemcpy(b->d_entries, entries.data(), entries.size() * sizeof(BatchEntry),
                          cudaMemcpyHostToDevice)) ||
        (err = cudaMalloc((void **)&b->d_items, std::max<size_t>(1, items.size()) * sizeof(BatchItem))) ||
        (!items.empty() &&
         (err = cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice))) ||
        (err = cudaMalloc((void **)&b->d_counters, kBuckets * sizeof(int))))
    {
        b->free_plan();
        return cuda_error(err, "fpg_batch_plan: work queue");
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
    b->grid = t.ctas_per_sm > 0 ? sms * t.ctas_per_sm : 1 << 30; // 0: capped by residency at launch
    b->tuning = t;
    b->planned = true;
    return FPG_OK;
}

// The launch sequence of a run: counter reset, one kernel per non-empty
// bucket, the split reduction and the contraction (outputs overwritten).
int launch_sequence(bool fp32, const fpg_batch_tuning &t, int grid_cap, const BatchEntry *d_entries,
                    const BatchItem *d_items, int *d_counters, const int *bucket_begin, int np, int64_t red_total,
                    int64_t con_total, cudaStream_t st)
{
    cudaError_t e;
    if ((e = cudaMemsetAsync(d_counters, 0, kBuckets * sizeof(int), st)))
        return cuda_error(e, "cudaMemsetAsync");
    const int sms = sm_count();
    for (int k = 0; k < kBuckets; ++k)
    {
        const int n_items = bucket_begin[k + 1] - bucket_begin[k];
        if (n_items <= 0)
            continue;
        int grid = -1; // item-grid form
        if (t.ctas_per_sm >= 0)
        {
            const int cap = sms * max_resident(fp32, k, t.threads_per_cta);
            grid = std::max(1, std::min({grid_cap, cap, n_items}));
        }
        if ((e = launch_bucket(fp32, k, grid, t.threads_per_cta, d_entries, d_items + bucket_begin[k], n_items,
                               d_counters + k, st)))
            return cuda_error(e, "persistent batch kernel");
    }
    const unsigned g1 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((red_total + 255) / 256, sms * 16));
    k_batch_reduce<<<g1, 256, 0, st>>>(d_entries, np, red_total);
    if ((e = launched()))
        return cuda_error(e, "batch reduction");
    const unsigned g2 = (unsigned)std::max<int64_t>(1, std::min<int64_t>((con_total + 255) / 256, sms * 16));
    if (fp32)
        k_batch_contract<float2><<<g2, 256, 0, st>>>(d_entries, np, con_total);
    else
        k_batch_contract<double2><<<g2, 256, 0, st>>>(d_entries, np, con_total);
    if ((e = launched()))
        return cuda_error(e, "batch contraction");
    return FPG_OK;
}

int do_run(fpg_batch *b, cudaStream_t st)
{
    return launch_sequence(b->dtype == FPG_C64, b->tuning, b->grid, b->d_entries, b->d_items, b->d_counters,
                           b->bucket_begin, (int)b->problems.size(), b->red_total, b->con_total, st);
}

} // namespace

namespace fpg
{
// Expectation problems run as one batch, stream-ordered: the work queue and
// the partial tables come from the library's pool on `st` and go back to it
// on `st` after the run, and the host arrays are uploaded with asynchronous
// copies, so nothing synchronises the device (the serving loop merges the
// small expectation requests it admits together this way).  Default tuning;
// outputs are overwritten.  A problem's result does not depend on the other
// problems of the run (every summation order is fixed per problem).
int run_merged_expect(int32_t dtype, const MergedExpect *probs, int n, cudaStream_t st)
{
    if (n <= 0)
        return FPG_OK;
    std::vector<fpg_batch::Problem> problems((size_t)n);
    for (int i = 0; i < n; ++i)
        problems[(size_t)i] = fpg_batch::Problem{probs[i].op, probs[i].coeffs, probs[i].n_operators,
                                                  probs[i].states, probs[i].out, probs[i].n_states};
    const bool fp32 = dtype == FPG_C64;
    const fpg_batch_tuning t{256, 0, 1 << 15, 40};
    HostPlan hp;
    if (int rc = plan_host(problems, fp32, t, hp))
        return rc;
    const size_t b_partial = (size_t)std::max<int64_t>(1, hp.partial_total) * sizeof(double);
    const size_t b_entries = hp.entries.size() * sizeof(BatchEntry);
    const size_t b_items = std::max<size_t>(1, hp.items.size()) * sizeof(BatchItem);
    const size_t b_counters = kBuckets * sizeof(int);
    auto al = [](size_t v) { return (v + 255) & ~size_t(255); };
    void *buf = nullptr;
    if (int rc = fpg_device_alloc(&buf, al(b_partial) + al(b_entries) + al(b_items) + b_counters, st))
        return rc;
    char *base = (char *)buf;
    double *d_partial = (double *)base;
    BatchEntry *d_entries = (BatchEntry *)(base + al(b_partial));
    BatchItem *d_items = (BatchItem *)(base + al(b_partial) + al(b_entries));
    int *d_counters = (int *)(base + al(b_partial) + al(b_entries) + al(b_items));
    for (size_t i = 0; i < hp.entries.size(); ++i)
        hp.entries[i].partial = d_partial + hp.partial_off[i];
    cudaError_t e;
    int rc = FPG_OK;
    // pageable sources: each copy has read its source when it returns
    if ((e = cudaMemcpyAsync(d_entries, hp.entries.data(), b_entries, cudaMemcpyHostToDevice, st)) ||
        (!hp.items.empty() &&
         (e = cudaMemcpyAsync(d_items, hp.items.data(), hp.items.size() * sizeof(BatchItem), cudaMemcpyHostToDevice,
                              st))))
        rc = cuda_error(e, "cudaMemcpyAsync (merged batch plan)");
    if (rc == FPG_OK)
        rc = launch_sequence(fp32, t, 1 << 30, d_entries, d_items, d_counters, hp.bucket_begin, n, hp.red_total,
                             hp.con_total, st);
    fpg_device_free(buf, st);
    return rc;
}

size_t merged_expect_scratch_bytes(const fpg_operator *op, int64_t S, const void *states, bool fp32)
{
    int32_t V = 1, TC = 1, n_splits = 1;
    entry_tiling(op, S, states, fp32, fpg_batch_tuning{256, 0, 1 << 15, 40}, V, TC, n_splits);
    const int64_t ctiles = (S + (int64_t)TC * V - 1) / ((int64_t)TC * V);
    const int64_t items = (int64_t)op->chunks.size() * ctiles * n_splits;
    return (size_t)(n_splits * op->P * S) * sizeof(double) + (size_t)items * sizeof(BatchItem) + sizeof(BatchEntry) +
           4 * 256 + kBuckets * sizeof(int);
}
} // namespace fpg

extern "C"
{

    int fpg_batch_create(int32_t dtype, fpg_batch **out)
    {
        if (!out)
            return set_error(FPG_ERR_INVALID, "out is null");
        *out = nullptr;
        if (dtype != FPG_C128 && dtype != FPG_C64)
            return set_error(FPG_ERR_INVALID, "dtype must be FPG_C128 or FPG_C64");
        fpg_batch *b = new (std::nothrow) fpg_batch();
        if (!b)
            return set_error(FPG_ERR_NOMEM, "host allocation failed");
        b->dtype = dtype;
        cudaError_t e = cudaGetDevice(&b->device);
        if (e != cudaSuccess)
        {
            delete b;
            return cuda_error(e, "cudaGetDevice");
        }
        *out = b;
        return FPG_OK;
    }

    int fpg_batch_add(fpg_batch *b, const fpg_operator *op, const void *coeffs, int64_t n_operators,
                      const void *states, void *out, int64_t n_states)
    {
        if (!b || !op)
            return set_error(FPG_ERR_INVALID, "null batch or operator");
        if (n_operators < 1 || n_states < 1)
            return set_error(FPG_ERR_INVALID, "n_operators and n_states must be >= 1");
        if (op->P < 1)
            return set_error(FPG_ERR_INVALID, "operator has no strings");
        if (!coeffs || !states || !out)
            return set_error(FPG_ERR_INVALID, "null array");
        const uintptr_t al = b->dtype == FPG_C64 ? 8 : 16;
        if ((uintptr_t)coeffs % al || (uintptr_t)states % al || (uintptr_t)out % al)
            return set_error(FPG_ERR_INVALID, "complex arrays must be aligned to their element size");
        if (op->device != b->device)
            return set_error(FPG_ERR_INVALID, "operator and batch live on different devices");
        b->problems.push_back(fpg_batch::Problem{op, coeffs, n_operators, states, out, n_states});
        b->free_plan();
        return FPG_OK;
    }

    int fpg_batch_plan(fpg_batch *b, const fpg_batch_tuning *tuning)
    {
        if (!b)
            return set_error(FPG_ERR_INVALID, "batch is null");
        if (b->problems.empty())
            return set_error(FPG_ERR_INVALID, "batch is empty");
        return do_plan(b, tuning ? *tuning : b->tuning);
    }

    int fpg_batch_run(fpg_batch *b, void *stream)
    {
        if (!b)
            return set_error(FPG_ERR_INVALID, "batch is null");
        if (!b->planned)
            if (int rc = fpg_batch_plan(b, nullptr))
                return rc;
        return do_run(b, (cudaStream_t)stream);
    }

    int fpg_batch_run_graph(fpg_batch *b, void *stream)
    {
        if (!b)
            return set_error(FPG_ERR_INVALID, "batch is null");
        if (!b->planned)
            if (int rc = fpg_batch_plan(b, nullptr))
                return rc;
        cudaStream_t st = (cudaStream_t)stream;
        cudaError_t e;
        if (!b->exec)
        {
            // capture on a private stream so a legacy-default caller stream works too
            cudaStream_t cap;
            if ((e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking)))
                return cuda_error(e, "cudaStreamCreate");
            if ((e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal)))
            {
                cudaStreamDestroy(cap);
                return cuda_error(e, "cudaStreamBeginCapture");
            }
            const int rc = do_run(b, cap);
            cudaGraph_t g = nullptr;
            e = cudaStreamEndCapture(cap, &g);
            cudaStreamDestroy(cap);
            if (rc != FPG_OK)
            {
                if (g)
                    cudaGraphDestroy(g);
                return rc;
            }
            if (e != cudaSuccess)
                return cuda_error(e, "cudaStreamEndCapture");
            if ((e = cudaGraphInstantiate(&b->exec, g, 0)))
            {
                cudaGraphDestroy(g);
                return cuda_error(e, "cudaGraphInstantiate");
            }
            b->graph = g;
        }
        if ((e = cudaGraphLaunch(b->exec, st)))
            return cuda_error(e, "cudaGraphLaunch");
        return FPG_OK;
    }

    int fpg_batch_autotune(fpg_batch *b, void *stream, fpg_batch_tuning *best, double *best_ms)
    {
        if (!b)
            return set_error(FPG_ERR_INVALID, "batch is null");
        if (b->problems.empty())
            return set_error(FPG_ERR_INVALID, "batch is empty");
        cudaStream_t st = (cudaStream_t)stream;
        // candidate grid: CTA size x residency x work-item granularity
        const int threads[] = {128, 256};
        const int ctas[] = {0, -1};
        const int rows[] = {1 << 15, 1 << 17};
        const int tiles[] = {16, 48};
        fpg_batch_tuning top{};
        double top_ms = 1e300;
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int th : threads)
            for (int cp : ctas)
                for (int rw : rows)
                    for (int tmb : tiles)
                {
                    const fpg_batch_tuning cand{th, cp, rw, tmb};
                    if (int rc = do_plan(b, cand))
                    {
                        cudaEventDestroy(e0);
                        cudaEventDestroy(e1);
                        return rc;
                    }
                    if (int rc = do_run(b, st)) // warm-up
                    {
                        cudaEventDestroy(e0);
                        cudaEventDestroy(e1);
                        return rc;
                    }
                    cudaEventRecord(e0, st);
                    const int reps = 2;
                    for (int r = 0; r < reps; ++r)
                        if (int rc = do_run(b, st))
                        {
                            cudaEventDestroy(e0);
                            cudaEventDestroy(e1);
                            return rc;
                        }
                    cudaEventRecord(e1, st);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    ms /= reps;
                    if (ms < top_ms)
                    {
                        top_ms = ms;
                        top = cand;
                    }
                }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (int rc = do_plan(b, top))
            return rc;
        if (best)
            *best = top;
        if (best_ms)
            *best_ms = top_ms;
        return FPG_OK;
    }

    int fpg_batch_info(const fpg_batch *b, int64_t *n_problems, int64_t *n_items, fpg_batch_tuning *tuning)
    {
        if (!b)
            return set_error(FPG_ERR_INVALID, "batch is null");
        if (n_problems)
            *n_problems = (int64_t)b->problems.size();
        if (n_items)
            *n_items = b->planned ? b->bucket_begin[kBuckets] : 0;
        if (tuning)
            *tuning = b->tuning;
        return FPG_OK;
    }

    int fpg_batch_destroy(fpg_batch *b)
    {
        if (!b)
            return FPG_OK;
        b->free_plan();
        delete b;
        return FPG_OK;
    }

} // extern "C"
