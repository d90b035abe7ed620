// capi.cpp -- the extern "C" entry points of libfpg.so (declared in include/fpg.h).
//
// Host side of the engine: argument checks (same conditions as the
// reference's std::invalid_argument checks), string encoding and x-grouping,
// launch planning, stream-ordered scratch memory and kernel dispatch.
#include "fpg.h"

#include <algorithm>
#include <atomic>
#include <initializer_list>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "common.cuh"
#include "host_internal.hpp"

using namespace fpg;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static thread_local std::string g_last_error;
static std::atomic<uint64_t> g_launches{0};

namespace fpg
{
cudaError_t launched()
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
    return cudaGetLastError();
}
int sm_count()
{
    constexpr int kMaxDev = 64;
    static std::atomic<int> cache[kMaxDev] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev)
        return 152;
    int v = cache[dev].load(std::memory_order_relaxed);
    if (v > 0)
        return v;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
        return 152;
    cache[dev].store(v, std::memory_order_relaxed);
    return v;
}
int set_error(int code, const std::string &msg)
{
    g_last_error = msg;
    return code;
}
int cuda_error(cudaError_t e, const char *where)
{
    return set_error(FPG_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
} // namespace fpg

#define FPG_CUDA(call)                                                                                                 \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t e_ = (call);                                                                                       \
        if (e_ != cudaSuccess)                                                                                         \
            return cuda_error(e_, #call);                                                                              \
    } while (0)

// ---------------------------------------------------------------------------
// operator encoding
// ---------------------------------------------------------------------------

namespace fpg
{

int encode_strings(const char *strings, int64_t P, int n, std::vector<StringRec> &recs, std::vector<int32_t> &orig,
                   std::vector<Group> &groups, std::vector<Chunk> &chunks, std::vector<int> &class_begin)
{
    std::vector<StringRec> raw((size_t)P);
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
        raw[(size_t)j] = StringRec{x, z, ml, ny & 3u};
    }
    std::vector<int32_t> idx((size_t)P);
    for (int64_t j = 0; j < P; ++j)
        idx[(size_t)j] = (int32_t)j;
    std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) {
        const StringRec &ra = raw[(size_t)a], &rb = raw[(size_t)b];
        if (ra.x != rb.x)
            return ra.x < rb.x;
        const uint32_t pa = ra.meta & 1u, pb = rb.meta & 1u;
        if (pa != pb)
            return pa < pb;
        return ra.z < rb.z;
    });
    recs.resize((size_t)P);
    orig.resize((size_t)P);
    for (int64_t s = 0; s < P; ++s)
    {
        recs[(size_t)s] = raw[(size_t)idx[(size_t)s]];
        orig[(size_t)s] = idx[(size_t)s];
    }
    groups.clear();
    for (int64_t s = 0; s < P;)
    {
        int64_t e = s;
        while (e < P && recs[(size_t)e].x == recs[(size_t)s].x)
            ++e;
        groups.push_back(Group{recs[(size_t)s].x, (int32_t)s, (int32_t)(e - s)});
        s = e;
    }
    // chunks of each group, bucketed by kernel class
    std::vector<std::vector<Chunk>> by_class(kNumChunkClasses);
    for (const Group &g : groups)
    {
        int32_t ev_b = g.begin, ev_e = g.begin;
        while (ev_e < g.begin + g.count && (recs[(size_t)ev_e].meta & 1u) == 0)
            ++ev_e;
        int32_t od_b = ev_e, od_e = g.begin + g.count;
        while (ev_b < ev_e || od_b < od_e)
        {
            const int ne = std::min<int32_t>(8, ev_e - ev_b);
            const int no = std::min<int32_t>(8, od_e - od_b);
            const int cls = chunk_class_for(ne, no);
            Chunk c{};
            c.x = g.x;
            c.begin_even = ev_b;
            c.begin_odd = od_b;
            c.n_even = (int16_t)ne;
            c.n_odd = (int16_t)no;
            by_class[(size_t)cls].push_back(c);
            ev_b += ne;
            od_b += no;
        }
    }
    chunks.clear();
    class_begin.assign(kNumChunkClasses + 1, 0);
    for (int c = 0; c < kNumChunkClasses; ++c)
    {
        class_begin[(size_t)c] = (int)chunks.size();
        chunks.insert(chunks.end(), by_class[(size_t)c].begin(), by_class[(size_t)c].end());
    }
    class_begin[kNumChunkClasses] = (int)chunks.size();
    return FPG_OK;
}

} // namespace fpg

namespace
{

struct DeviceGuard
{
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess)
        {
            ok = false;
            return;
        }
        if (prev != dev && cudaSetDevice(dev) != cudaSuccess)
            ok = false;
    }
    ~DeviceGuard()
    {
        if (prev >= 0)
            cudaSetDevice(prev);
    }
};

template <typename T> cudaError_t upload(T **dptr, const std::vector<T> &v)
{
    *dptr = nullptr;
    if (v.empty())
        return cudaSuccess;
    cudaError_t e = cudaMalloc((void **)dptr, v.size() * sizeof(T));
    if (e != cudaSuccess)
        return e;
    return cudaMemcpy(*dptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
}

void free_dev(fpg_operator *op)
{
    cudaFree(op->d_recs);
    cudaFree(op->d_orig);
    cudaFree(op->d_groups);
    cudaFree(op->d_chunks);
    cudaFree(op->d_fast_chunks);
    cudaFree(op->d_wht);
    cudaFree(op->d_pairs);
    op->d_pairs = nullptr;
    cudaFree(op->d_tiles);
    op->d_tiles = nullptr;
    cudaFree(op->d_tile_pairs);
    op->d_tile_pairs = nullptr;
    cudaFree(op->d_margs);
    op->d_margs = nullptr;
    cudaFree(op->d_local);
    op->d_local = nullptr;
    cudaFree(op->d_glob);
    op->d_glob = nullptr;
    op->d_recs = nullptr;
    op->d_orig = nullptr;
    op->d_groups = nullptr;
    op->d_chunks = nullptr;
    op->d_fast_chunks = nullptr;
    op->d_wht = nullptr;
}

// The tile family: pair-kernel groups x = 2^a + 2^b (a < b) whose z' lie in
// {0, 2^a}, gathered into units of four row bits Q with up to six groups
// whose both bits lie in Q (k_expect_tile.cu).  Greedy cover: up to
// kTileMaxCoverQubits qubits each unit is the set of four bits that covers
// the most groups left (all 153 pairs of 18 qubits: 29 units; the lower
// bound is 27); above it the first group left opens a unit and its other two
// bits are the ones that bring the most groups left into it (32 units for
// the same pairs; 18 for the 91 pairs of 14 qubits either way, which is
// optimal).  Taken groups leave op->pairs for op->tiles /
// op->tile_pairs and is_wht 4.  Operators on fewer than kTileMinQubits
// qubits, or with fewer than kTileMinGroups such groups, keep the pair kernel.
constexpr int kTileMinQubits = 8;
constexpr int kTileMinGroups = 6;
constexpr int kTileMaxCoverQubits = 24; // C(24, 4) = 10626 candidate sets per unit

void build_tiles(fpg_operator *op, const std::vector<size_t> &pair_groups, std::vector<char> &is_wht)
{
    const int n = op->n;
    if (n < kTileMinQubits || n > 63)
        return;
    // at[a * n + b]: the eligible group on bits a < b, or -1
    std::vector<int64_t> at((size_t)n * (size_t)n, -1);
    std::vector<int> abit_of(op->groups.size(), -1);
    int left = 0;
    for (size_t k = 0; k < pair_groups.size(); ++k)
    {
        const PairChunk &pc = op->pairs[k];
        if (__builtin_popcountll(pc.x) != 2)
            continue;
        const int a = __builtin_ctzll(pc.x), b = 63 - __builtin_clzll(pc.x);
        if (pc.abit != -1 && pc.abit != a)
            continue;
        at[(size_t)a * n + b] = (int64_t)pair_groups[k];
        abit_of[pair_groups[k]] = pc.abit;
        ++left;
    }
    if (left < kTileMinGroups)
        return;
    static const int si[kTileSlots] = {0, 0, 1, 0, 1, 2};
    static const int sj[kTileSlots] = {1, 2, 2, 3, 3, 3};
    auto cell = [&](int x, int y) -> int64_t & { return x < y ? at[(size_t)x * n + y] : at[(size_t)y * n + x]; };
    size_t scan = 0;
    while (left > 0)
    {
        int q[4];
        if (n <= kTileMaxCoverQubits)
        {
            // the set of four row bits that covers the most groups left (the
            // first such set in lexicographic order)
            int best = -1;
            for (int a = 0; a < n; ++a)
                for (int b = a + 1; b < n; ++b)
                {
                    const int ab = cell(a, b) >= 0;
                    for (int c = b + 1; c < n; ++c)
                    {
                        const int abc = ab + (cell(a, c) >= 0) + (cell(b, c) >= 0);
                        for (int d = c + 1; d < n; ++d)
                        {
                            const int cnt = abc + (cell(a, d) >= 0) + (cell(b, d) >= 0) + (cell(c, d) >= 0);
                            if (cnt > best)
                            {
                                best = cnt;
                                q[0] = a;
                                q[1] = b;
                                q[2] = c;
                                q[3] = d;
                            }
                        }
                    }
                }
        }
        else
        {
            while (at[scan] < 0)
                ++scan;
            const int a = (int)(scan / (size_t)n), b = (int)(scan % (size_t)n);
            int best = -1, bc = -1, bd = -1;
            for (int c = 0; c < n; ++c)
            {
                if (c == a || c == b)
                    continue;
                for (int d = c + 1; d < n; ++d)
                {
                    if (d == a || d == b)
                        continue;
                    const int qq[4] = {a, b, c, d};
                    int cnt = 0;
                    for (int i = 0; i < 4; ++i)
                        for (int j = i + 1; j < 4; ++j)
                            cnt += cell(qq[i], qq[j]) >= 0;
                    if (cnt > best)
                    {
                        best = cnt;
                        bc = c;
                        bd = d;
                    }
                }
            }
            q[0] = a;
            q[1] = b;
            q[2] = bc;
            q[3] = bd;
            std::sort(q, q + 4);
        }
        TileChunk t{};
        for (int k = 0; k < 4; ++k)
            t.q[k] = (int8_t)q[k];
        for (int s = 0; s < kTileSlots; ++s)
        {
            int64_t &g = cell(q[si[s]], q[sj[s]]);
            if (g < 0)
                continue;
            const Group &grp = op->groups[(size_t)g];
            t.begin[s] = grp.begin;
            t.count[s] = (int8_t)grp.count;
            op->tile_pairs.push_back(PairChunk{grp.x, grp.begin, grp.count, abit_of[(size_t)g], 0});
            is_wht[(size_t)g] = 4;
            g = -1;
            --left;
        }
        op->tiles.push_back(t);
    }
    std::vector<PairChunk> rest;
    for (size_t k = 0; k < pair_groups.size(); ++k)
        if (is_wht[pair_groups[k]] == 2)
            rest.push_back(op->pairs[k]);
    op->pairs.swap(rest);
}

// Per-call decomposition of the x-groups, by the signs z' (z with the pairing
// bit dropped) of their strings:
//   all z' in {0, e_a}, <= kPairMaxStrings strings   -> pair kernel;
//   every z' of <= 1 bit, >= kMargMinStrings strings -> marginal kernel;
//   >= kWhtMinStrings strings                        -> transform kernel;
//   the rest -> direct-kernel chunks bucketed by class.
void build_fast_decomposition(fpg_operator *op)
{
    op->wht.clear();
    op->wht_max_count = 0;
    op->wht_both = false;
    op->pairs.clear();
    op->tiles.clear();
    op->tile_pairs.clear();
    op->margs.clear();
    op->marg_max_high = 0;
    std::vector<std::vector<Chunk>> by_class(kNumChunkClasses);
    std::vector<char> is_wht(op->groups.size(), 0); // 1: transform, 2: pair, 3: marginal, 4: tile kernel
    std::vector<size_t> pair_groups;
    for (size_t gi = 0; gi < op->groups.size(); ++gi)
    {
        const Group &g = op->groups[gi];
        // signs with the pairing bit (top bit of x) dropped: z' of each string
        const uint64_t pbit = g.x ? (1ull << (63 - __builtin_clzll(g.x))) : 0ull;
        uint64_t bits = 0; // union of the z'
        bool single = true; // every z' has at most one bit
        int flags = 0;
        for (int32_t s = g.begin; s < g.begin + g.count; ++s)
        {
            const StringRec &r = op->recs[(size_t)s];
            bits |= r.z & ~pbit;
            single = single && __builtin_popcountll(r.z & ~pbit) <= 1;
            flags |= (r.meta & 1u) ? 2 : 1;
        }
        if (g.count <= kPairMaxStrings && __builtin_popcountll(bits) <= 1)
        {
            // pair kernel: every z' in {0, e_a}
            is_wht[gi] = 2;
            op->pairs.push_back(PairChunk{g.x, g.begin, g.count, bits ? __builtin_ctzll(bits) : -1, 0});
            pair_groups.push_back(gi);
            continue;
        }
        const int high = __builtin_popcountll(bits & ~31ull);
        if (single && g.count >= kMargMinStrings && high <= kMargMaxHighBits)
        {
            // marginal kernel: every z' in {0} u {e_b}
            is_wht[gi] = 3;
            op->margs.push_back(MargChunk{g.x, bits, g.begin, g.count, flags, 0});
            op->marg_max_high = std::max(op->marg_max_high, high);
            continue;
        }
        if (g.count < kWhtMinStrings)
            continue; // direct kernel
        is_wht[gi] = 1;
        int32_t n_even_total = 0;
        while (n_even_total < g.count && (op->recs[(size_t)(g.begin + n_even_total)].meta & 1u) == 0)
            ++n_even_total;
        for (int32_t b = 0; b < g.count; b += kWhtMaxStrings)
        {
            const int32_t cnt = std::min<int32_t>(kWhtMaxStrings, g.count - b);
            const int32_t ne = std::max<int32_t>(0, std::min<int32_t>(cnt, n_even_total - b));
            op->wht.push_back(WhtChunk{g.x, g.begin + b, (int16_t)cnt, (int16_t)ne});
            op->wht_max_count = std::max(op->wht_max_count, (int)cnt);
            op->wht_both = op->wht_both || (ne > 0 && ne < cnt);
        }
    }
    build_tiles(op, pair_groups, is_wht);
    // direct chunks of the remaining groups, in the order of the full decomposition
    for (int c = 0; c < kNumChunkClasses; ++c)
        for (int i = op->class_begin[(size_t)c]; i < op->class_begin[(size_t)c + 1]; ++i)
        {
            const Chunk &ch = op->chunks[(size_t)i];
            // the chunk's group: the one containing its first string
            const int32_t first = ch.n_even > 0 ? ch.begin_even : ch.begin_odd;
            const auto it = std::upper_bound(op->groups.begin(), op->groups.end(), first,
                                             [](int32_t v, const Group &g) { return v < g.begin; });
            const size_t gi = (size_t)(it - op->groups.begin()) - 1;
            if (!is_wht[gi])
                by_class[(size_t)c].push_back(ch);
        }
    op->fast_chunks.clear();
    op->fast_class_begin.assign(kNumChunkClasses + 1, 0);
    for (int c = 0; c < kNumChunkClasses; ++c)
    {
        op->fast_class_begin[(size_t)c] = (int)op->fast_chunks.size();
        op->fast_chunks.insert(op->fast_chunks.end(), by_class[(size_t)c].begin(), by_class[(size_t)c].end());
    }
    op->fast_class_begin[kNumChunkClasses] = (int)op->fast_chunks.size();

    // family-local string order (each family may write its own partial table)
    static const int fam_of[5] = {kFamDirect, kFamWht, kFamPair, kFamMarg, kFamTile}; // by is_wht value
    op->local.assign((size_t)op->P, 0);
    op->glob.clear();
    op->glob.reserve((size_t)op->P);
    for (int f = 0; f < kNumFam; ++f)
    {
        op->fam_begin[f] = (int64_t)op->glob.size();
        for (size_t gi = 0; gi < op->groups.size(); ++gi)
        {
            if (fam_of[(int)is_wht[gi]] != f)
                continue;
            const Group &g = op->groups[gi];
            for (int32_t s = g.begin; s < g.begin + g.count; ++s)
            {
                op->local[(size_t)s] = (int32_t)((int64_t)op->glob.size() - op->fam_begin[f]);
                op->glob.push_back(op->orig[(size_t)s]);
            }
        }
    }
    op->fam_begin[kNumFam] = (int64_t)op->glob.size();
}

int check_dtype(int32_t dtype)
{
    if (dtype != FPG_C128 && dtype != FPG_C64)
        return set_error(FPG_ERR_INVALID, "dtype must be FPG_C128 or FPG_C64");
    return FPG_OK;
}

// Complex arrays are read with vector loads of one element (16 B complex128,
// 8 B complex64); a misaligned pointer is an argument error, never a fault.
int check_aligned(int32_t dtype, std::initializer_list<const void *> ptrs)
{
    const uintptr_t a = dtype == FPG_C64 ? 8 : 16;
    for (const void *p : ptrs)
        if (p && ((uintptr_t)p % a) != 0)
            return set_error(FPG_ERR_INVALID, "complex arrays must be aligned to their element size");
    return FPG_OK;
}

// Device memory of the library's temporaries: one stream-ordered pool per
// device that keeps up to FPG_POOL_KEEP_BYTES (default 4 GiB) mapped across
// synchronisations.  The device's default pool gives all freed memory back
// at every synchronisation, so host-buffer calls that synchronise would map
// and unmap their staging and scratch buffers (hundreds of MB) every time.
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxPoolDevices];

uint64_t pool_keep_bytes()
{
    const char *e = std::getenv("FPG_POOL_KEEP_BYTES");
    if (e && *e)
    {
        char *end = nullptr;
        const unsigned long long v = std::strtoull(e, &end, 10);
        if (end && *end == '\0')
            return v;
    }
    return 4ull << 30;
}

cudaError_t library_pool(cudaMemPool_t *out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return e;
    if (dev < 0 || dev >= kMaxPoolDevices)
        return cudaDeviceGetDefaultMemPool(out, dev);
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pools[dev])
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t p = nullptr;
        if ((e = cudaMemPoolCreate(&p, &props)) != cudaSuccess)
            return e;
        uint64_t keep = pool_keep_bytes();
        if ((e = cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep)) != cudaSuccess)
        {
            cudaMemPoolDestroy(p);
            return e;
        }
        g_pools[dev] = p;
    }
    *out = g_pools[dev];
    return cudaSuccess;
}

cudaError_t pool_alloc(void **p, size_t bytes, cudaStream_t st)
{
    cudaMemPool_t pool = nullptr;
    cudaError_t e = library_pool(&pool);
    if (e != cudaSuccess)
        return e;
    return cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, st);
}

// Stream-ordered scratch allocation, freed on scope exit (also stream ordered).
struct Scratch
{
    void *p = nullptr;
    cudaStream_t st;
    explicit Scratch(cudaStream_t s) : st(s)
    {
    }
    cudaError_t alloc(size_t bytes)
    {
        return pool_alloc(&p, bytes, st);
    }
    ~Scratch()
    {
        if (p)
            cudaFreeAsync(p, st);
    }
};

int pick_tc(int64_t lanes)
{
    int tc = 1;
    while (tc < 32 && tc < lanes)
        tc <<= 1;
    return tc;
}

ExpectPlan plan_expect(const fpg_operator *op, int64_t S, bool fp32, const void *psi)
{
    ExpectPlan p{};
    p.V = (fp32 && (S % 2 == 0) && (((uintptr_t)psi) % 16 == 0)) ? 2 : 1;
    const int64_t lanes = (S + p.V - 1) / p.V;
    p.TC = column_lanes_for_l2(pick_tc(lanes), op->n, p.V * (fp32 ? 8 : 16), kColumnTileBytes);
    p.n_ctiles = (int)((S + (int64_t)p.TC * p.V - 1) / ((int64_t)p.TC * p.V));
    p.wht_TC = column_lanes_for_l2(pick_tc(S), op->n, fp32 ? 8 : 16, kColumnTileBytes);
    p.wht_ctiles = (int)((S + p.wht_TC - 1) / p.wht_TC);
    const int64_t NB = op->n >= 5 ? ((int64_t)1 << (op->n - 5)) : 1;    // 32-row blocks
    const int64_t NB16 = op->n >= 4 ? ((int64_t)1 << (op->n - 4)) : 1;  // 16-row blocks (transform kernel)
    const bool over = column_tile_footprint(p.TC, op->n, p.V * (fp32 ? 8 : 16)) > kColumnTileBytes;
    const bool over1 = column_tile_footprint(p.wht_TC, op->n, fp32 ? 8 : 16) > kColumnTileBytes;
    // row splits of one launch: enough CTAs for kSplitCtasPerSm per SM, an L2
    // row window when even a one-line column tile does not fit, >= 4 blocks
    // per row lane.  The double-float kernels are issue-bound and gain from
    // fewer, longer CTAs (less epilogue and reduction per row); the float32
    // ones are bound by load latency and gain from more CTAs to pick from
    // (float32 marginal kernel, mixed n=18 step: 6.92 / 6.84 / 6.93 / 7.08 ms
    // at 6 / 12 / 24 / 48 CTAs per SM; transform kernel: 7.04 / 6.98 / 6.93 /
    // 6.95 ms at 8 / 12 / 24 / 48)
    constexpr int kSplitCtasPerSmF64 = 4, kSplitCtasPerSmF32 = 24;
    constexpr int kSplitCtasPerSmF32Marg = 12, kSplitCtasPerSmF32Wht = 24;
    // (float64, n=14 weight<=2 step: marginal kernel 2.156 / 2.044 / 2.108 /
    // 2.128 ms at 2 / 4 / 8 / 16 CTAs per SM; transform kernel 2.100 / 2.044 /
    // 2.048 ms at 2 / 4 / 8)
    constexpr int kSplitCtasPerSmF64Marg = 4, kSplitCtasPerSmF64Wht = 4;
    const int per_sm_all = fp32 ? kSplitCtasPerSmF32 : kSplitCtasPerSmF64;
    // min_rounds: blocks per row lane each split keeps at least (4; the
    // transform kernel 1: its CTAs do little per-CTA work besides the rows,
    // and at a narrow call's few column tiles 4 rounds left most SMs idle --
    // n=14 weight<=2, 128 states: 64 CTAs on 152 SMs, 63.5 us per launch)
    auto pick_at = [](int per_sm, int64_t ctas_per_split, int64_t blocks, int row_lanes, bool windowed,
                      int64_t window, int min_rounds = 4) {
        if (ctas_per_split <= 0)
            return 1;
        const int64_t target = (int64_t)sm_count() * per_sm;
        int64_t s = (target + ctas_per_split - 1) / ctas_per_split;
        if (windowed)
            s = std::max<int64_t>(s, (blocks + window - 1) / window);
        const int64_t mx = std::max<int64_t>(1, blocks / ((int64_t)row_lanes * min_rounds));
        return (int)std::max<int64_t>(1, std::min<int64_t>(std::min(s, mx), 65535));
    };
    auto pick = [&](int64_t ctas_per_split, int64_t blocks, int row_lanes, bool windowed, int64_t window) {
        return pick_at(per_sm_all, ctas_per_split, blocks, row_lanes, windowed, window);
    };
    p.fam_splits[kFamDirect] =
        pick((int64_t)op->fast_chunks.size() * p.n_ctiles, NB / 2, 256 / p.TC, over, kWindowBlocks);
    p.fam_splits[kFamPair] = pick((int64_t)op->pairs.size() * p.n_ctiles, NB / 2, 256 / p.TC, over, kWindowBlocks);
    p.fam_splits[kFamMarg] = pick_at(fp32 ? kSplitCtasPerSmF32Marg : kSplitCtasPerSmF64Marg,
                                     (int64_t)op->margs.size() * p.wht_ctiles, NB / 2, 256 / p.wht_TC, over1,
                                     kWindowBlocks);
    p.fam_splits[kFamWht] = pick_at(fp32 ? kSplitCtasPerSmF32Wht : kSplitCtasPerSmF64Wht,
                                    (int64_t)op->wht.size() * p.wht_ctiles, NB16 / 2, kWhtThreads / p.wht_TC, over1,
                                    2 * kWindowBlocks, 1);
    // the tile kernel: one element per lane (the V = 1 tiling), its column
    // tile within the L2 budget (its units read rows spread over the whole
    // state), the df64 copy of the state for the float64 path
    p.tile_kernel = !op->tiles.empty() && !over1 && op->n >= 4 &&
                    (fp32 || ((int64_t)1 << op->n) * S * 16 <= kDfSplitMaxBytes);
    p.tile_TC = p.wht_TC;
    p.tile_ctiles = p.wht_ctiles;
    p.fam_splits[kFamTile] =
        p.tile_kernel ? pick((int64_t)op->tiles.size() * p.tile_ctiles, NB16, 256 / p.tile_TC, false, 0)
                      : pick((int64_t)op->tile_pairs.size() * p.n_ctiles, NB / 2, 256 / p.TC, over, kWindowBlocks);
    p.n_splits = 1;
    for (int f = 0; f < kNumFam; ++f)
        p.n_splits = std::max(p.n_splits, p.fam_splits[f]);
    return p;
}

// Scratch (doubles) of the families' partial tables; off[f] = offset of
// family f's table, or -1 when it writes the caller-ordered table directly.
int64_t family_partials(const fpg_operator *op, const ExpectPlan &plan, int64_t S, int64_t (&off)[kNumFam])
{
    int64_t total = 0;
    for (int f = 0; f < kNumFam; ++f)
    {
        const int64_t Pf = op->fam_begin[f + 1] - op->fam_begin[f];
        off[f] = -1;
        if (plan.fam_splits[f] > 1 && Pf > 0)
        {
            off[f] = total;
            total += (int64_t)plan.fam_splits[f] * Pf * S;
        }
    }
    return total;
}

// A second stream forked from st (after all of st's work so far) and joined
// back into it: per caller stream (per thread for the per-thread and legacy
// default handles), one non-blocking stream of the same priority, created on
// first use and kept.  Without a fork (or when no side stream can be had)
// stream() is st itself.
class SideStream
{
  public:
    SideStream(cudaStream_t st, bool fork) : st_(st)
    {
        if (!fork || !(side_ = side_for(st)))
            return;
        if (cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&join_, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventRecord(fork_, st) != cudaSuccess || cudaStreamWaitEvent(side_, fork_, 0) != cudaSuccess)
        {
            cudaGetLastError();
            side_ = nullptr;
        }
    }
    ~SideStream()
    {
        join();
        if (fork_)
            cudaEventDestroy(fork_);
        if (join_)
            cudaEventDestroy(join_);
    }
    cudaStream_t stream() const
    {
        return side_ ? side_ : st_;
    }
    // st waits for everything queued on the side stream (idempotent)
    cudaError_t join()
    {
        if (!side_ || joined_)
            return cudaSuccess;
        joined_ = true;
        cudaError_t e = cudaEventRecord(join_, side_);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(st_, join_, 0);
        return e;
    }

  private:
    static cudaStream_t make_like(cudaStream_t st)
    {
        int prio = 0;
        cudaStream_t s = nullptr;
        if (cudaStreamGetPriority(st, &prio) != cudaSuccess ||
            cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio) != cudaSuccess)
        {
            cudaGetLastError();
            return nullptr;
        }
        return s;
    }
    static cudaStream_t side_for(cudaStream_t st)
    {
        // the per-thread and legacy default handles name a different stream
        // in every thread (or one shared by all): a side stream per thread
        if (st == cudaStreamPerThread || st == nullptr || st == cudaStreamLegacy)
        {
            thread_local cudaStream_t mine[2] = {nullptr, nullptr};
            cudaStream_t &s = mine[st == cudaStreamPerThread ? 0 : 1];
            if (!s)
                s = make_like(st);
            return s;
        }
        static std::mutex mu;
        static std::vector<std::pair<cudaStream_t, cudaStream_t>> map;
        std::lock_guard<std::mutex> lock(mu);
        for (auto &kv : map)
            if (kv.first == st)
                return kv.second;
        if (map.size() >= 64)
            return nullptr;
        cudaStream_t s = make_like(st);
        if (s)
            map.emplace_back(st, s);
        return s;
    }
    cudaStream_t st_;
    cudaStream_t side_ = nullptr;
    cudaEvent_t fork_ = nullptr, join_ = nullptr;
    bool joined_ = false;
};

// The apply stage.  float32 as is; float64 in df64 on the float32 pipes:
// state and coefficients split once (and range-checked) into df64 copies,
// the df64 kernel, then the float64 kernel, which returns at once unless a
// value lay outside the df64 range (the df64 kernel then did nothing).
// n_cw: complex coefficients in cw (P, or P * S when weighted).
size_t apply_scratch_bytes(int n, int64_t S, int64_t n_cw, bool fp32)
{
    const int64_t n_elem = ((int64_t)1 << n) * S;
    if (fp32 || n_elem * 16 > kDfSplitMaxBytes)
        return 0;
    // flag, the column maxima of the states and of the coefficients, the
    // df64 copies
    return 256 + 2 * df_split_colmax_bytes(S) + (size_t)n_elem * 16 + (size_t)n_cw * 16;
}

// The group-diagonal table of a plain apply (launch_group_diag) in bytes, or
// 0 where the kernels sum each group's strings in registers: apply_weighted
// (its diagonals differ per column), fewer than 4 columns or fewer than two
// strings per group on average (the table saves little), or a table above
// kDiagTableMaxBytes.  The table (16 bytes per group and row in df64, 8 in
// float32) replaces, per column, one signed sum over the group's strings.
constexpr size_t kDiagTableMaxBytes = size_t(1) << 30;
size_t diag_table_bytes(const DevOp &dop, int64_t S, bool weighted, bool fp32)
{
    if (weighted || S < 4 || dop.G <= 0 || dop.P < 2 * dop.G)
        return 0;
    const size_t b = ((size_t)dop.G << dop.n) * (fp32 ? 8 : 16);
    return b <= kDiagTableMaxBytes ? b : 0;
}

// Scratch for `base` bytes and, when `tab` > 0, a table after them at a
// 256-byte offset (returned in *diag).  Without room for the table, `tab` is
// dropped (the kernels then sum in registers) rather than failing the call.
cudaError_t alloc_with_table(Scratch &sc, size_t base, size_t tab, void **diag)
{
    *diag = nullptr;
    const size_t off = (base + 255) & ~size_t(255);
    if (tab)
    {
        if (sc.alloc(off + tab) == cudaSuccess)
        {
            *diag = (char *)sc.p + off;
            return cudaSuccess;
        }
        cudaGetLastError();
        sc.p = nullptr;
    }
    return base ? sc.alloc(base) : cudaSuccess;
}

// cw: n_cw = P coefficients (one column) or, weighted, (P, S) per column
int run_apply(bool fp32, bool weighted, const DevOp &dop, const void *cw, int64_t n_cw, const void *states, void *out,
              int64_t S, cudaStream_t st)
{
    const size_t bytes = apply_scratch_bytes(dop.n, S, n_cw, fp32);
    Scratch sc(st);
    void *diag = nullptr;
    if (bytes == 0)
    {
        // float32 (or a float64 state too large for its df64 copy)
        if (fp32)
        {
            FPG_CUDA(alloc_with_table(sc, 0, diag_table_bytes(dop, S, weighted, true), &diag));
            if (diag)
                FPG_CUDA(launch_group_diag(false, dop, cw, diag, nullptr, st));
        }
        FPG_CUDA(launch_apply(fp32, weighted, dop, cw, states, out, S, st, nullptr, diag));
        return FPG_OK;
    }
    FPG_CUDA(alloc_with_table(sc, bytes, diag_table_bytes(dop, S, weighted, false), &diag));
    int *flag = (int *)sc.p;
    void *cm_psi = (char *)sc.p + 256;
    void *cm_cw = (char *)cm_psi + df_split_colmax_bytes(S);
    void *psi_df = (char *)cm_cw + df_split_colmax_bytes(S);
    void *cw_df = (char *)psi_df + (((int64_t)1 << dop.n) * S) * 16;
    const int64_t cw_cols = (weighted && S > 0 && n_cw % S == 0) ? S : 1;
    FPG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
    FPG_CUDA(launch_df_split(states, (int64_t)1 << dop.n, S, psi_df, cm_psi, flag, st));
    FPG_CUDA(launch_df_split(cw, n_cw / cw_cols, cw_cols, cw_df, cm_cw, flag, st));
    if (diag)
        FPG_CUDA(launch_group_diag(true, dop, cw_df, diag, flag, st));
    FPG_CUDA(launch_apply_df(weighted, dop, cw_df, psi_df, out, S, flag, st, diag));
    FPG_CUDA(launch_apply(false, weighted, dop, cw, states, out, S, st, flag));
    return FPG_OK;
}

int run_expect_strings(const fpg_operator *op, const void *psi, double *ev, int64_t S, bool fp32, cudaStream_t st)
{
    if (S <= 0 || op->P <= 0)
        return FPG_OK;
    const ExpectPlan plan = plan_expect(op, S, fp32, psi);
    int64_t off[kNumFam];
    const int64_t scratch = family_partials(op, plan, S, off);
    // scratch: the df64 range flag of the float64 path (see df64.cuh) and the
    // families' partial tables
    const bool need_flag =
        !fp32 && (!op->pairs.empty() || !op->tiles.empty() || !op->margs.empty() || !op->wht.empty());
    // (the flag, then the column maxima of the df64 range check)
    const size_t flag_bytes = need_flag ? 256 + df_split_colmax_bytes(S) : 0;
    Scratch partial(st);
    if (scratch > 0 || need_flag)
        FPG_CUDA(partial.alloc(flag_bytes + (size_t)scratch * sizeof(double)));
    int *range_flag = need_flag ? (int *)partial.p : nullptr;
    if (need_flag)
        FPG_CUDA(cudaMemsetAsync(range_flag, 0, sizeof(int), st));
    double *partials = (double *)((char *)partial.p + flag_bytes);
    // float64 path: the state split into df64 once (same size), when it fits;
    // otherwise the kernels split it themselves and the pass only checks the
    // columns' range
    Scratch split(st);
    const int64_t n_elem = ((int64_t)1 << op->n) * S;
    if (need_flag)
    {
        void *colmax = (char *)partial.p + 256;
        if (n_elem * 16 <= kDfSplitMaxBytes)
            FPG_CUDA(split.alloc((size_t)n_elem * 16));
        FPG_CUDA(launch_df_split(psi, (int64_t)1 << op->n, S, split.p, colmax, range_flag, st));
    }
    const void *psi_df = split.p;
    // family f writes ev directly (caller order) or its own partial table
    // (family-local order, reduced below)
    auto target = [&](int f, DevOp &d, ExpectPlan &pl) -> double * {
        d = op->dev();
        pl = plan;
        pl.n_splits = plan.fam_splits[f];
        if (off[f] < 0)
            return ev;
        d.orig = op->d_local;
        d.P = op->fam_begin[f + 1] - op->fam_begin[f];
        return partials + off[f];
    };
    DevOp d;
    ExpectPlan pl;
    // the transform and marginal families run on a side stream, concurrently
    // with the pair and direct families on st: their CTAs fill the SMs that
    // the other kernels' last waves leave idle (every family writes its own
    // strings' rows)
    SideStream side(st, (!op->pairs.empty() || !op->tiles.empty()) && (!op->wht.empty() || !op->margs.empty()));
    const cudaStream_t st2 = side.stream();
    if (!op->wht.empty())
    {
        double *dst = target(kFamWht, d, pl);
        FPG_CUDA(launch_expect_wht(fp32, psi, S, op->n, d, op->d_wht, (int)op->wht.size(), op->wht_max_count,
                                   op->wht_both, pl.wht_TC, pl.wht_ctiles, pl.n_splits, dst, range_flag, psi_df, st2));
        if (off[kFamWht] >= 0)
            FPG_CUDA(launch_reduce_family(partials + off[kFamWht], plan.fam_splits[kFamWht],
                                          op->fam_begin[kFamWht + 1] - op->fam_begin[kFamWht], S,
                                          op->d_glob + op->fam_begin[kFamWht], ev, st2));
    }
    if (!op->margs.empty())
    {
        double *dst = target(kFamMarg, d, pl);
        FPG_CUDA(launch_expect_marg(fp32, psi, S, op->n, d, op->d_margs, (int)op->margs.size(), op->marg_max_high,
                                    pl.wht_TC, pl.wht_ctiles, pl.n_splits, dst, range_flag, psi_df, st2));
        if (off[kFamMarg] >= 0)
            FPG_CUDA(launch_reduce_family(partials + off[kFamMarg], plan.fam_splits[kFamMarg],
                                          op->fam_begin[kFamMarg + 1] - op->fam_begin[kFamMarg], S,
                                          op->d_glob + op->fam_begin[kFamMarg], ev, st2));
    }
    if (!op->tiles.empty())
    {
        double *dst = target(kFamTile, d, pl);
        if (plan.tile_kernel)
        {
            FPG_CUDA(launch_expect_tile(fp32, fp32 ? psi : psi_df, S, op->n, d, op->d_tiles, (int)op->tiles.size(),
                                        plan.tile_TC, plan.tile_ctiles, pl.n_splits, dst, st));
            if (!fp32)
                FPG_CUDA(launch_expect_pair_f64_if(psi, S, op->n, d, op->d_tile_pairs, (int)op->tile_pairs.size(), pl,
                                                   dst, range_flag, st));
        }
        else
            FPG_CUDA(launch_expect_pair(fp32, psi, S, op->n, d, op->d_tile_pairs, (int)op->tile_pairs.size(), pl, dst,
                                        range_flag, psi_df, st));
    }
    if (!op->pairs.empty())
    {
        double *dst = target(kFamPair, d, pl);
        FPG_CUDA(launch_expect_pair(fp32, psi, S, op->n, d, op->d_pairs, (int)op->pairs.size(), pl, dst, range_flag,
                                    psi_df, st));
    }
    {
        double *dst = target(kFamDirect, d, pl);
        for (int c = 0; c < kNumChunkClasses; ++c)
        {
            const int b = op->fast_class_begin[(size_t)c], e = op->fast_class_begin[(size_t)c + 1];
            if (e > b)
                FPG_CUDA(launch_expect_chunks(fp32, psi, S, op->n, d, op->d_fast_chunks + b, e - b, c, pl, dst, st));
        }
    }
    for (int f = 0; f < kNumFam; ++f)
        if (off[f] >= 0 && f != kFamWht && f != kFamMarg)
            FPG_CUDA(launch_reduce_family(partials + off[f], plan.fam_splits[f],
                                          op->fam_begin[f + 1] - op->fam_begin[f], S, op->d_glob + op->fam_begin[f],
                                          ev, st));
    FPG_CUDA(side.join());
    return FPG_OK;
}

} // namespace

namespace fpg
{
// Upper bound of the stream-ordered scratch one fpg_summed_expect (weighted =
// false) or fpg_summed_apply_weighted (weighted = true) call draws.
size_t request_scratch_bytes(const fpg_operator *op, int64_t K, int64_t S, bool fp32, bool weighted)
{
    const size_t P = (size_t)op->P;
    if (weighted)
    {
        const size_t csz = fp32 ? 8 : 16;
        size_t b = 2 * P * (size_t)S * csz + apply_scratch_bytes(op->n, S, op->P * S, fp32);
        if (fp32)
            b += tc_workspace_bytes(2 * op->P, S, K);
        return b + 4096;
    }
    const ExpectPlan plan = plan_expect(op, S, fp32, nullptr);
    int64_t off[kNumFam];
    size_t b = P * (size_t)S * sizeof(double) + (size_t)family_partials(op, plan, S, off) * sizeof(double) + 512 +
               df_split_colmax_bytes(S);
    const int64_t split_bytes = ((int64_t)1 << op->n) * S * 16;
    if (!fp32 && (!op->pairs.empty() || !op->tiles.empty() || !op->margs.empty() || !op->wht.empty()) &&
        split_bytes <= kDfSplitMaxBytes)
        b += (size_t)split_bytes; // the df64 copy of the state
    b += fp32 ? tc_workspace_bytes(2 * K, S, op->P) : oz_workspace_bytes(2 * K, S, op->P);
    return b + 4096;
}
} // namespace fpg

// ---------------------------------------------------------------------------
// entry points
// ---------------------------------------------------------------------------

extern "C"
{

    int fpg_abi_version(void)
    {
        return FPG_ABI_VERSION;
    }

    const char *fpg_last_error(void)
    {
        return g_last_error.c_str();
    }

    int fpg_device_error(int *code, void *stream)
    {
        if (!code)
            return set_error(FPG_ERR_INVALID, "code is null");
        FPG_CUDA(read_device_error(code, (cudaStream_t)stream));
        return FPG_OK;
    }

    int fpg_kernel_launches(uint64_t *total)
    {
        if (!total)
            return set_error(FPG_ERR_INVALID, "total is null");
        *total = g_launches.load(std::memory_order_relaxed);
        return FPG_OK;
    }

    int fpg_device_count(int *count)
    {
        if (!count)
            return set_error(FPG_ERR_INVALID, "count is null");
        int c = 0;
        cudaError_t e = cudaGetDeviceCount(&c);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            c = 0;
        }
        *count = c;
        return FPG_OK;
    }

    int fpg_device_alloc(void **ptr, size_t bytes, void *stream)
    {
        if (!ptr)
            return set_error(FPG_ERR_INVALID, "ptr is null");
        *ptr = nullptr;
        cudaError_t e = pool_alloc(ptr, bytes, (cudaStream_t)stream);
        if (e == cudaErrorMemoryAllocation)
        {
            cudaGetLastError();
            return set_error(FPG_ERR_NOMEM, "device memory exhausted (" + std::to_string(bytes) + " bytes)");
        }
        FPG_CUDA(e);
        return FPG_OK;
    }

    int fpg_device_free(void *ptr, void *stream)
    {
        if (ptr)
            FPG_CUDA(cudaFreeAsync(ptr, (cudaStream_t)stream));
        return FPG_OK;
    }

    int fpg_release_cached_memory(void)
    {
        std::lock_guard<std::mutex> lock(g_pool_mu);
        for (cudaMemPool_t p : g_pools)
            if (p)
                FPG_CUDA(cudaMemPoolTrimTo(p, 0));
        return FPG_OK;
    }

    int fpg_pointer_is_device(const void *ptr, int *is_device)
    {
        if (!is_device)
            return set_error(FPG_ERR_INVALID, "is_device is null");
        *is_device = 0;
        if (!ptr)
            return FPG_OK;
        cudaPointerAttributes a{};
        cudaError_t e = cudaPointerGetAttributes(&a, ptr);
        if (e != cudaSuccess)
        {
            cudaGetLastError();
            return FPG_OK;
        }
        *is_device = (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? 1 : 0;
        return FPG_OK;
    }

    int fpg_operator_create(const char *strings, int64_t n_strings, int32_t n_qubits, fpg_operator **out)
    {
        if (!out)
            return set_error(FPG_ERR_INVALID, "out is null");
        *out = nullptr;
        if (n_strings < 0)
            return set_error(FPG_ERR_INVALID, "n_strings must be >= 0");
        if (n_strings > 0 && !strings)
            return set_error(FPG_ERR_INVALID, "strings is null");
        if (n_qubits < 1 || n_qubits > 40)
            return set_error(FPG_ERR_UNSUPPORTED, "n_qubits must be in [1, 40]");
        if (n_strings > (int64_t)0x7fffffff)
            return set_error(FPG_ERR_UNSUPPORTED, "too many strings");
        fpg_operator *op = new (std::nothrow) fpg_operator();
        if (!op)
            return set_error(FPG_ERR_NOMEM, "host allocation failed");
        op->n = n_qubits;
        op->P = n_strings;
        int rc = encode_strings(strings, n_strings, n_qubits, op->recs, op->orig, op->groups, op->chunks,
                                op->class_begin);
        if (rc != FPG_OK)
        {
            delete op;
            return rc;
        }
        cudaError_t e = cudaGetDevice(&op->device);
        if (e == cudaSuccess)
            e = upload(&op->d_recs, op->recs);
        if (e == cudaSuccess)
            e = upload(&op->d_orig, op->orig);
        if (e == cudaSuccess)
            e = upload(&op->d_groups, op->groups);
        if (e == cudaSuccess)
            e = upload(&op->d_chunks, op->chunks);
        build_fast_decomposition(op);
        if (e == cudaSuccess)
            e = upload(&op->d_fast_chunks, op->fast_chunks);
        if (e == cudaSuccess)
            e = upload(&op->d_wht, op->wht);
        if (e == cudaSuccess)
            e = upload(&op->d_pairs, op->pairs);
        if (e == cudaSuccess)
            e = upload(&op->d_tiles, op->tiles);
        if (e == cudaSuccess)
            e = upload(&op->d_tile_pairs, op->tile_pairs);
        if (e == cudaSuccess)
            e = upload(&op->d_margs, op->margs);
        if (e == cudaSuccess)
            e = upload(&op->d_local, op->local);
        if (e == cudaSuccess)
            e = upload(&op->d_glob, op->glob);
        if (e != cudaSuccess)
        {
            free_dev(op);
            delete op;
            return cuda_error(e, "fpg_operator_create");
        }
        *out = op;
        return FPG_OK;
    }

    int fpg_operator_destroy(fpg_operator *op)
    {
        if (!op)
            return FPG_OK;
        {
            DeviceGuard g(op->device);
            free_dev(op);
        }
        delete op;
        return FPG_OK;
    }

    int fpg_operator_info(const fpg_operator *op, int32_t *n_qubits, int64_t *n_strings, int64_t *n_groups)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (n_qubits)
            *n_qubits = op->n;
        if (n_strings)
            *n_strings = op->P;
        if (n_groups)
            *n_groups = (int64_t)op->groups.size();
        return FPG_OK;
    }

    int fpg_operator_family_stats(const fpg_operator *op, int64_t *row_visits, int64_t *sign_adds)
    {
        if (!op || !row_visits || !sign_adds)
            return set_error(FPG_ERR_INVALID, "null argument");
        // the per-call decomposition, by kernel family
        const int64_t D = (int64_t)1 << op->n;
        for (int f = 0; f < FPG_FAMILY_COUNT; ++f)
            row_visits[f] = sign_adds[f] = 0;
        for (int c = 0; c < kNumChunkClasses; ++c)
            for (int i = op->fast_class_begin[(size_t)c]; i < op->fast_class_begin[(size_t)c + 1]; ++i)
            {
                const bool paired = (op->fast_chunks[(size_t)i].x >> 5) != 0;
                const int64_t rows = paired ? D / 2 : D;
                row_visits[FPG_FAMILY_DIRECT] += rows;
                sign_adds[FPG_FAMILY_DIRECT] += rows * (kChunkClasses[c].ge + kChunkClasses[c].go);
            }
        for (const WhtChunk &w : op->wht)
        {
            const bool paired = (w.x >> 4) != 0;
            const int64_t rows = paired ? D / 2 : D;
            const int parts = (w.n_even > 0 ? 1 : 0) + (w.n_even < w.count ? 1 : 0);
            row_visits[FPG_FAMILY_TRANSFORM] += rows;
            // 16-point transform: 4 adds per row per part; one add per string per 16 rows
            sign_adds[FPG_FAMILY_TRANSFORM] += rows * 4 * parts + (rows / 16) * w.count;
        }
        // four FMAs per row, the running sums included: no sign adds
        for (const PairChunk &pc : op->pairs)
            row_visits[FPG_FAMILY_PAIR] += pc.x != 0 ? D / 2 : D; // rows paired across or inside 32-row blocks
        for (const PairChunk &pc : op->tile_pairs)
            row_visits[FPG_FAMILY_TILE] += pc.x != 0 ? D / 2 : D;
        for (const MargChunk &mc : op->margs)
        {
            const int64_t rows = mc.x != 0 ? D / 2 : D;
            const int parts = ((mc.flags & 1) ? 1 : 0) + ((mc.flags & 2) ? 1 : 0);
            row_visits[FPG_FAMILY_MARGINAL] += rows;
            sign_adds[FPG_FAMILY_MARGINAL] += rows * parts * 17 / 8; // marginal tree: 68 adds per 32 rows and part
        }
        return FPG_OK;
    }

    int fpg_operator_stats(const fpg_operator *op, int64_t *n_chunks, int64_t *row_visits, int64_t *sign_adds)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        int64_t v[FPG_FAMILY_COUNT], a[FPG_FAMILY_COUNT];
        fpg_operator_family_stats(op, v, a);
        int64_t visits = 0, adds = 0;
        for (int f = 0; f < FPG_FAMILY_COUNT; ++f)
        {
            visits += v[f];
            adds += a[f];
        }
        if (n_chunks)
            *n_chunks = (int64_t)(op->fast_chunks.size() + op->wht.size() + op->pairs.size() + op->tiles.size() +
                                  op->margs.size());
        if (row_visits)
            *row_visits = visits;
        if (sign_adds)
            *sign_adds = adds;
        return FPG_OK;
    }

    int fpg_sparse_repr(const char *string, int32_t n_qubits, uint64_t *cols, void *vals, void *stream)
    {
        if (!string || !cols || !vals)
            return set_error(FPG_ERR_INVALID, "null argument");
        if (n_qubits < 1 || n_qubits > 40)
            return set_error(FPG_ERR_UNSUPPORTED, "n_qubits must be in [1, 40]");
        std::vector<StringRec> recs;
        std::vector<int32_t> orig;
        std::vector<Group> groups;
        std::vector<Chunk> chunks;
        std::vector<int> cb;
        int rc = encode_strings(string, 1, n_qubits, recs, orig, groups, chunks, cb);
        if (rc != FPG_OK)
            return rc;
        FPG_CUDA(launch_sparse_repr(recs[0].x, recs[0].z, (int)(recs[0].meta & 3u), n_qubits, cols, vals,
                                    (cudaStream_t)stream));
        return FPG_OK;
    }

    int fpg_expect_strings(const fpg_operator *op, const void *states, double *ev, int64_t n_states, int32_t dtype,
                           void *stream)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_states < 0)
            return set_error(FPG_ERR_INVALID, "n_states must be >= 0");
        if (n_states > 0 && op->P > 0 && (!states || !ev))
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {states}))
            return rc;
        if ((uintptr_t)ev % 8 != 0)
            return set_error(FPG_ERR_INVALID, "ev must be 8-byte aligned");
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        return run_expect_strings(op, states, ev, n_states, dtype == FPG_C64, (cudaStream_t)stream);
    }

    int fpg_summed_expect(const fpg_operator *op, const void *coeffs, int64_t n_operators, const void *states,
                          void *out, int64_t n_states, int32_t dtype, void *stream)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_states < 0 || n_operators < 0)
            return set_error(FPG_ERR_INVALID, "n_states and n_operators must be >= 0");
        if (n_states == 0 || n_operators == 0 || op->P == 0)
            return FPG_OK;
        if (!coeffs || !states || !out)
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {coeffs, states, out}))
            return rc;
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        cudaStream_t st = (cudaStream_t)stream;
        const bool fp32 = dtype == FPG_C64;
        // per-string table, then (float64) the contraction's flag
        Scratch evb(st);
        const size_t ev_bytes = ((size_t)op->P * (size_t)n_states * sizeof(double) + 255) & ~(size_t)255;
        FPG_CUDA(evb.alloc(ev_bytes + 256));
        int *flag = (int *)((char *)evb.p + ev_bytes);
        Scratch ws(st);
        if (!fp32)
        {
            // float64: the H half of the contraction's preparation runs on a
            // side stream while the per-string stage computes
            FPG_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), st));
            FPG_CUDA(ws.alloc(oz_workspace_bytes(2 * n_operators, n_states, op->P)));
            SideStream side(st, true);
            FPG_CUDA(launch_contract_oz_prep_h(coeffs, op->P, n_operators, n_states, ws.p, flag, side.stream()));
            if (int rc = run_expect_strings(op, states, (double *)evb.p, n_states, fp32, st))
                return rc;
            FPG_CUDA(side.join());
        }
        else if (int rc = run_expect_strings(op, states, (double *)evb.p, n_states, fp32, st))
            return rc;
        if (fp32)
        {
            // mixed path: 3xTF32 contraction on the tensor cores
            FPG_CUDA(ws.alloc(tc_workspace_bytes(2 * n_operators, n_states, op->P)));
            FPG_CUDA(launch_contract_tc_expect(coeffs, (const double *)evb.p, op->P, n_operators, n_states, out,
                                               ws.p, st));
            return FPG_OK;
        }
        // float64: the contraction on the tensor cores (exact digit-slice
        // products), or the float64 GEMM when H or E holds a non-finite value
        FPG_CUDA(launch_contract_oz_expect(coeffs, (const double *)evb.p, op->P, n_operators, n_states, out, ws.p,
                                           flag, st));
        FPG_CUDA(launch_contract_f64_if(coeffs, (const double *)evb.p, op->P, n_operators, n_states, out, flag, st));
        return FPG_OK;
    }

    int fpg_apply(const fpg_operator *op, const void *coeffs, const void *states, void *out, int64_t n_states,
                  int32_t dtype, void *stream)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_states < 0)
            return set_error(FPG_ERR_INVALID, "n_states must be >= 0");
        if (n_states == 0 || op->P == 0)
            return FPG_OK;
        if (!coeffs || !states || !out)
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {coeffs, states, out}))
            return rc;
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        cudaStream_t st = (cudaStream_t)stream;
        const bool fp32 = dtype == FPG_C64;
        const size_t csz = fp32 ? 8 : 16;
        Scratch cw(st);
        FPG_CUDA(cw.alloc((size_t)op->P * csz));
        const DevOp dop = op->dev();
        FPG_CUDA(launch_prep_coeffs(fp32, dop, coeffs, 0, cw.p, st));
        return run_apply(fp32, false, dop, cw.p, op->P, states, out, n_states, st);
    }

    int fpg_summed_apply(const fpg_operator *op, const void *coeffs, int64_t n_operators, const void *states,
                         void *out, int64_t n_states, int32_t dtype, void *stream)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_states < 0 || n_operators < 0)
            return set_error(FPG_ERR_INVALID, "n_states and n_operators must be >= 0");
        if (n_states == 0 || op->P == 0 || n_operators == 0)
            return FPG_OK;
        if (!coeffs || !states || !out)
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {coeffs, states, out}))
            return rc;
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        cudaStream_t st = (cudaStream_t)stream;
        const bool fp32 = dtype == FPG_C64;
        const size_t csz = fp32 ? 8 : 16;
        Scratch cw(st);
        FPG_CUDA(cw.alloc((size_t)op->P * csz));
        const DevOp dop = op->dev();
        FPG_CUDA(launch_prep_coeffs(fp32, dop, coeffs, n_operators, cw.p, st));
        return run_apply(fp32, false, dop, cw.p, op->P, states, out, n_states, st);
    }

    int fpg_summed_apply_weighted(const fpg_operator *op, const void *coeffs, int64_t n_operators,
                                  const void *states, const void *data, void *out, int64_t n_states, int32_t dtype,
                                  void *stream)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_states < 0 || n_operators < 0)
            return set_error(FPG_ERR_INVALID, "n_states and n_operators must be >= 0");
        if (n_states == 0 || op->P == 0 || n_operators == 0)
            return FPG_OK;
        if (!coeffs || !states || !out || !data)
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {coeffs, states, out}))
            return rc;
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        cudaStream_t st = (cudaStream_t)stream;
        const bool fp32 = dtype == FPG_C64;
        const size_t csz = fp32 ? 8 : 16;
        const DevOp dop = op->dev();
        Scratch w(st), cw(st);
        FPG_CUDA(w.alloc((size_t)op->P * (size_t)n_states * csz));
        FPG_CUDA(cw.alloc((size_t)op->P * (size_t)n_states * csz));
        if (fp32)
        {
            // mixed path: weighted coefficients with the 3xTF32 tensor-core GEMM
            Scratch ws(st);
            FPG_CUDA(ws.alloc(tc_workspace_bytes(2 * op->P, n_states, n_operators)));
            FPG_CUDA(launch_weighted_tc(coeffs, (const float *)data, op->P, n_operators, n_states, w.p, ws.p, st));
        }
        else
            FPG_CUDA(launch_weighted_coeffs(fp32, coeffs, data, op->P, n_operators, n_states, w.p, st));
        FPG_CUDA(launch_prep_weighted(fp32, dop, w.p, n_states, cw.p, st));
        return run_apply(fp32, true, dop, cw.p, op->P * n_states, states, out, n_states, st);
    }

    int fpg_to_tensor(const fpg_operator *op, const void *coeffs, int64_t n_operators, void *out, int32_t dtype,
                      void *stream)
    {
        if (!op)
            return set_error(FPG_ERR_INVALID, "op is null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_operators < 0)
            return set_error(FPG_ERR_INVALID, "n_operators must be >= 0");
        if (n_operators == 0 || op->P == 0)
            return FPG_OK;
        if (!coeffs || !out)
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {coeffs, out}))
            return rc;
        if (op->n > 24)
            return set_error(FPG_ERR_UNSUPPORTED, "to_tensor: 2^n x 2^n matrices only up to n = 24");
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        FPG_CUDA(launch_to_tensor(dtype == FPG_C64, op->dev(), coeffs, n_operators, out, (cudaStream_t)stream));
        return FPG_OK;
    }

    int fpg_op_product(const fpg_operator *a, const void *coeffs_a, const fpg_operator *b, const void *coeffs_b,
                       uint64_t *out_x, uint64_t *out_z, void *out_coeffs, int64_t *n_out, void *stream)
    {
        if (!a || !b || !n_out)
            return set_error(FPG_ERR_INVALID, "a, b and n_out must not be null");
        *n_out = 0;
        const int64_t Pa = a->P, Pb = b->P;
        if (Pa == 0 || Pb == 0)
            return FPG_OK;
        if (a->n != b->n)
            return set_error(FPG_ERR_INVALID, "Mismatched dimensions for provided PauliOp");
        if (a->device != b->device)
            return set_error(FPG_ERR_INVALID, "the operators live on different devices");
        if (!coeffs_a || !coeffs_b || !out_x || !out_z || !out_coeffs)
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(FPG_C128, {coeffs_a, coeffs_b, out_coeffs}))
            return rc;
        if (Pa * Pb >= ((int64_t)1 << 31))
            return set_error(FPG_ERR_UNSUPPORTED, "too many string pairs (n_strings(a) * n_strings(b) >= 2^31)");
        DeviceGuard g(a->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        cudaStream_t st = (cudaStream_t)stream;
        Scratch ws(st);
        FPG_CUDA(ws.alloc(product_workspace_bytes(Pa, Pb)));
        FPG_CUDA(launch_op_product(a->dev(), coeffs_a, b->dev(), coeffs_b, a->n, ws.p, out_x, out_z, out_coeffs, n_out,
                                   st));
        return FPG_OK;
    }

    int fpg_summed_square(const fpg_operator *op, const void *coeffs, int64_t n_operators, const fpg_operator *sq,
                          void *out, int32_t dtype, void *stream)
    {
        if (!op || !sq)
            return set_error(FPG_ERR_INVALID, "op and sq must not be null");
        if (int rc = check_dtype(dtype))
            return rc;
        if (n_operators < 0)
            return set_error(FPG_ERR_INVALID, "n_operators must be >= 0");
        const int64_t P = op->P, A = sq->P, K = n_operators;
        if (P > 0 && A > 0 && op->n != sq->n)
            return set_error(FPG_ERR_INVALID, "op and sq must act on the same number of qubits");
        if (A == 0 || K == 0)
            return FPG_OK;
        if (!out || (P > 0 && !coeffs))
            return set_error(FPG_ERR_INVALID, "null array");
        if (int rc = check_aligned(dtype, {coeffs, out}))
            return rc;
        if (square_max_terms(P) > ((int64_t)1 << 31))
            return set_error(FPG_ERR_UNSUPPORTED, "too many strings to square");
        DeviceGuard g(op->device);
        if (!g.ok)
            return set_error(FPG_ERR_CUDA, "cannot select the operator's device");
        cudaStream_t st = (cudaStream_t)stream;
        const bool fp32 = dtype == FPG_C64;
        if (P == 0)
        {
            FPG_CUDA(cudaMemsetAsync(out, 0, (size_t)A * (size_t)K * (fp32 ? 8 : 16), st));
            FPG_CUDA(cudaStreamSynchronize(st));
            return FPG_OK;
        }
        Scratch ws(st);
        FPG_CUDA(ws.alloc(square_workspace_bytes(P, A)));
        unsigned long long *d_found = nullptr;
        FPG_CUDA(launch_square(fp32, op->dev(), sq->dev(), coeffs, K, out, ws.p, &d_found, st));
        unsigned long long found = 0;
        FPG_CUDA(cudaMemcpyAsync(&found, d_found, sizeof(found), cudaMemcpyDeviceToHost, st));
        FPG_CUDA(cudaStreamSynchronize(st));
        if (found != (unsigned long long)P * (unsigned long long)P)
            return set_error(FPG_ERR_INVALID, "a product of two strings is not among the squared strings");
        return FPG_OK;
    }

} // extern "C"
