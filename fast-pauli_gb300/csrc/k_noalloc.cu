// k_noalloc.cu -- fpg_summed_expect_noalloc: SummedPauliOp expectation values
// for callers that cannot allocate device memory.
//
// Who needs this: code that runs inside a framework which has already
// reserved (nearly) all device memory for its own pool -- an XLA-style
// runtime that pre-allocates most of the GPU, or a PyTorch process held at
// its memory cap -- where a cudaMalloc either fails outright or would have to
// be negotiated with an allocator this library does not see; and
// latency-bound service loops that forbid allocation on the request path,
// because an allocation can block or synchronise the device and adds jitter.
// fpg_summed_expect draws its scratch (the encoded strings and the
// (n_strings x n_states) table of per-string expectation values) from the
// stream-ordered pool; this entry point instead uses one file-scope
// __device__ array of kNoallocScratchBytes, which every GPU that loads
// libfpg.so holds until the process exits.  The caller still owns and passes
// coefficients, states and the output.
//
// Set-up: the first call on each device resolves the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it for the
// life of the process; a cudaDeviceReset invalidates that address, so the
// entry point is not for processes that reset the device.  All calls share
// the one array, so calls whose GPU work overlaps (different streams,
// different host threads) race on it: order them on one stream or
// synchronise between them.  The host-side staging arrays are static too and
// are guarded by a mutex; the encoding is copied from them with pageable
// copies, which have read their source when cudaMemcpyAsync returns.  A copy
// recorded into a graph would instead read the arrays when the graph is
// replayed, after later calls have overwritten them, so a call made while
// its stream is being captured is refused (FPG_ERR_UNSUPPORTED).
//
// Work layout: one CTA per (chunk of up to 8 strings of an x-group, column
// tile), rows not split, so an operator of only a few strings on a large
// state (say under ten strings at n >= 24) runs on a few CTAs and is much
// slower than fpg_summed_expect, which splits the rows into partial tables.
#include <algorithm>
#include <cstring>
#include <mutex>

#include "fpg.h"

#include "common.cuh"
#include "host_internal.hpp"

namespace fpg
{
namespace
{

constexpr size_t kNoallocScratchBytes = size_t(16) << 20; // 16 MiB per device
constexpr int64_t kNoallocMaxStrings = 8192;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_mu;
void *g_scratch_addr[kMaxDevices] = {};

// host staging, static (no heap)
StringRec h_raw[kNoallocMaxStrings];
StringRec h_recs[kNoallocMaxStrings];
int32_t h_orig[kNoallocMaxStrings];
Group h_groups[kNoallocMaxStrings];
Chunk h_chunks[2 * kNoallocMaxStrings];
int h_chunk_cls[2 * kNoallocMaxStrings];
Chunk h_sorted_chunks[2 * kNoallocMaxStrings];

size_t align256(size_t v)
{
    return (v + 255) & ~size_t(255);
}

// Encode into the static host arrays: same records, order, groups and chunk
// classes as the pooled path's encoder.
int encode_static(const char *strings, int64_t P, int n, int64_t *G_out, int64_t *C_out, int *class_begin)
{
    for (int64_t j = 0; j < P; ++j)
    {
        uint64_t x = 0, z = 0;
        uint32_t ny = 0;
        for (int q = 0; q < n; ++q)
        {
            const char c = strings[j * n + q];
            const uint64_t bit = 1ull << (n - 1 - q);
            switch (c)
            {
            case 'I': break;
            case 'X': x |= bit; break;
            case 'Y': x |= bit; z |= bit; ++ny; break;
            case 'Z': z |= bit; break;
            default:
                return set_error(FPG_ERR_INVALID, std::string("Invalid Pauli character ") + c);
            }
        }
        uint32_t ml = 0;
        for (uint32_t r = 0; r < 32; ++r)
            ml |= (uint32_t)(__builtin_popcountll((uint64_t)r & z & 31ull) & 1) << r;
        h_raw[j] = StringRec{x, z, ml, ny & 3u};
        h_orig[j] = (int32_t)j;
    }
    // total order (x, parity of #Y, z, caller index): std::sort allocates nothing
    std::sort(h_orig, h_orig + P, [](int32_t a, int32_t b) {
        const StringRec &ra = h_raw[a], &rb = h_raw[b];
        if (ra.x != rb.x)
            return ra.x < rb.x;
        if ((ra.meta & 1u) != (rb.meta & 1u))
            return (ra.meta & 1u) < (rb.meta & 1u);
        if (ra.z != rb.z)
            return ra.z < rb.z;
        return a < b;
    });
    for (int64_t s = 0; s < P; ++s)
        h_recs[s] = h_raw[h_orig[s]];
    int64_t G = 0, C = 0;
    for (int64_t s = 0; s < P;)
    {
        int64_t e = s;
        while (e < P && h_recs[e].x == h_recs[s].x)
            ++e;
        h_groups[G++] = Group{h_recs[s].x, (int32_t)s, (int32_t)(e - s)};
        s = e;
    }
    for (int64_t g = 0; g < G; ++g)
    {
        const Group gr = h_groups[g];
        int32_t ev_b = gr.begin, ev_e = gr.begin;
        while (ev_e < gr.begin + gr.count && (h_recs[ev_e].meta & 1u) == 0)
            ++ev_e;
        int32_t od_b = ev_e, od_e = gr.begin + gr.count;
        while (ev_b < ev_e || od_b < od_e)
        {
            const int ne = std::min<int32_t>(8, ev_e - ev_b);
            const int no = std::min<int32_t>(8, od_e - od_b);
            Chunk c{};
            c.x = gr.x;
            c.begin_even = ev_b;
            c.begin_odd = od_b;
            c.n_even = (int16_t)ne;
            c.n_odd = (int16_t)no;
            h_chunk_cls[C] = chunk_class_for(ne, no);
            h_chunks[C++] = c;
            ev_b += ne;
            od_b += no;
        }
    }
    // bucket by class, keeping group order inside a class
    int64_t k = 0;
    for (int cls = 0; cls < kNumChunkClasses; ++cls)
    {
        class_begin[cls] = (int)k;
        for (int64_t i = 0; i < C; ++i)
            if (h_chunk_cls[i] == cls)
                h_sorted_chunks[k++] = h_chunks[i];
    }
    class_begin[kNumChunkClasses] = (int)k;
    *G_out = G;
    *C_out = C;
    return FPG_OK;
}

} // namespace
} // namespace fpg

using namespace fpg;

extern "C" int fpg_summed_expect_noalloc(const char *strings, int64_t n_strings, int32_t n_qubits,
                                         const void *coeffs, int64_t n_operators, const void *states, void *out,
                                         int64_t n_states, int32_t dtype, void *stream)
{
    if (dtype != FPG_C128 && dtype != FPG_C64)
        return set_error(FPG_ERR_INVALID, "dtype must be FPG_C128 or FPG_C64");
    if (n_qubits < 1 || n_qubits > 40)
        return set_error(FPG_ERR_UNSUPPORTED, "n_qubits must be in [1, 40]");
    if (n_strings < 0 || n_operators < 0 || n_states < 0)
        return set_error(FPG_ERR_INVALID, "sizes must be >= 0");
    if (n_strings == 0 || n_operators == 0 || n_states == 0)
        return FPG_OK;
    if (!strings || !coeffs || !states || !out)
        return set_error(FPG_ERR_INVALID, "null argument");
    const uintptr_t al = dtype == FPG_C64 ? 8 : 16;
    if ((uintptr_t)coeffs % al || (uintptr_t)states % al || (uintptr_t)out % al)
        return set_error(FPG_ERR_INVALID, "complex arrays must be aligned to their element size");
    if (n_strings > kNoallocMaxStrings)
        return set_error(FPG_ERR_INVALID, "fpg_summed_expect_noalloc: n_strings " + std::to_string(n_strings) +
                                              " exceeds the limit of " + std::to_string(kNoallocMaxStrings));
    const int64_t P = n_strings, S = n_states;
    // scratch layout: records | caller index | groups | chunks | ev table (P x S float64)
    const size_t off_recs = 0;
    const size_t off_orig = align256(off_recs + (size_t)P * sizeof(StringRec));
    const size_t off_groups = align256(off_orig + (size_t)P * sizeof(int32_t));
    const size_t off_chunks = align256(off_groups + (size_t)P * sizeof(Group));
    const size_t off_ev = align256(off_chunks + (size_t)(2 * P) * sizeof(Chunk));
    if ((double)P * (double)S * 8.0 + (double)off_ev > (double)kNoallocScratchBytes)
        return set_error(FPG_ERR_INVALID,
                         "fpg_summed_expect_noalloc: n_strings x n_states = " + std::to_string(P * S) +
                             " needs more than the " + std::to_string(kNoallocScratchBytes >> 20) +
                             " MiB static scratch (at most about " +
                             std::to_string(((int64_t)kNoallocScratchBytes - (int64_t)off_ev) / 8) + " values)");

    cudaStream_t st = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cap);
    if (e != cudaSuccess)
        return cuda_error(e, "cudaStreamIsCapturing");
    if (cap != cudaStreamCaptureStatusNone)
        return set_error(FPG_ERR_UNSUPPORTED, "fpg_summed_expect_noalloc: the stream is being captured; the encoding "
                                              "is copied from host arrays that the next call overwrites");

    std::lock_guard<std::mutex> lock(g_mu);
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(FPG_ERR_UNSUPPORTED, "device ordinal beyond the supported range");
    if (!g_scratch_addr[dev])
    {
        // once per device, with that device current
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return cuda_error(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_addr[dev] = p;
    }
    unsigned char *base = (unsigned char *)g_scratch_addr[dev];

    int64_t G = 0, C = 0;
    int class_begin[kNumChunkClasses + 1];
    if (int rc = encode_static(strings, P, n_qubits, &G, &C, class_begin))
        return rc;

    // pageable-source copies: each returns once the source has been staged,
    // so the static host arrays may be reused by the next call
    if ((e = cudaMemcpyAsync(base + off_recs, h_recs, (size_t)P * sizeof(StringRec), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(base + off_orig, h_orig, (size_t)P * sizeof(int32_t), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(base + off_groups, h_groups, (size_t)G * sizeof(Group), cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(base + off_chunks, h_sorted_chunks, (size_t)C * sizeof(Chunk), cudaMemcpyHostToDevice,
                             st)))
        return cuda_error(e, "cudaMemcpyAsync (staging the encoding)");
    double *ev = (double *)(base + off_ev);
    // every (string, state) entry is written by the expectation kernels; the
    // clear only guarantees that nothing can depend on a previous call's table
    if ((e = cudaMemsetAsync(ev, 0, (size_t)P * (size_t)S * sizeof(double), st)))
        return cuda_error(e, "cudaMemsetAsync");

    const bool fp32 = dtype == FPG_C64;
    ExpectPlan plan{};
    plan.V = (fp32 && (S % 2 == 0) && (((uintptr_t)states) % 16 == 0)) ? 2 : 1;
    const int64_t lanes = (S + plan.V - 1) / plan.V;
    plan.TC = 1;
    while (plan.TC < 32 && plan.TC < lanes)
        plan.TC <<= 1;
    plan.n_ctiles = (int)((S + (int64_t)plan.TC * plan.V - 1) / ((int64_t)plan.TC * plan.V));
    plan.n_splits = 1; // no partial-sum table: the ev table is the only scratch
    const DevOp dop{n_qubits, P, G, (const StringRec *)(base + off_recs), (const int32_t *)(base + off_orig),
                    (const Group *)(base + off_groups)};
    const Chunk *d_chunks = (const Chunk *)(base + off_chunks);
    for (int c = 0; c < kNumChunkClasses; ++c)
    {
        const int b = class_begin[c], en = class_begin[c + 1];
        if (en > b && (e = launch_expect_chunks(fp32, states, S, n_qubits, dop, d_chunks + b, en - b, c, plan, ev, st)))
            return cuda_error(e, "expectation kernel");
    }
    if ((e = launch_contract_real(fp32, coeffs, fp32, ev, P, n_operators, S, out, st)))
        return cuda_error(e, "contraction kernel");
    return FPG_OK;
}
