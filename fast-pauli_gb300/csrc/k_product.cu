// k_product.cu -- PauliOp products with equal strings merged, on the GPU.
//
// Replaces PauliOp operator* (fast_pauli/cpp/include/__pauli_op.hpp:237-281):
//     (sum_i a_i A_i)(sum_j b_j B_j) = sum_k c_k C_k
// over the distinct strings C_k among the products A_i B_j.  In the (x, z)
// encoding a product is a bit operation: A_i B_j = i^e C(x_i ^ x_j, z_i ^ z_j)
// with e = |x_i & z_i| + |x_j & z_j| - |x & z| + 2 |z_i & x_j| (mod 4)
// (sigma(x, z) = i^{x.z} X^x Z^z per qubit and Z X = -X Z).  The reference
// fills one hash map per OpenMP thread and concatenates them (equal strings
// found by different threads stay separate; the order is the maps' iteration
// order).  Here:
//
//  * every pair index p = i * Pb + j is sorted by its product key (x, z) with
//    a stable LSD radix sort on 4-bit digits (per pass: block histograms, an
//    exclusive scan in (digit, block) order, a scatter that ranks equal
//    digits by warp match masks, so the order of equal keys is the pair
//    order); the key is recomputed from p at each pass, so only 4-byte pair
//    indices move;
//  * runs of equal keys are flagged and numbered by an exclusive scan;
//  * one thread per run adds its products in pair order.
//
// The result lists each distinct string once, ordered by (x, z), with
// deterministic coefficient sums.
#include "common.cuh"

namespace fpg
{
namespace
{

constexpr int kRsThreads = 256, kRsRounds = 8, kRsTile = kRsThreads * kRsRounds; // items per block and pass
constexpr int kScanThreads = 1024, kScanPer = 4, kScanTile = kScanThreads * kScanPer;

// ------------------------------------------------------------------ scan
// exclusive prefix sums of int32 arrays, three kernels: tile-local scans with
// tile totals, one block over the totals, tile offsets added back

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t *warp_tot, int32_t &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const int32_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o)
            inc += y;
    }
    if (lane == 31)
        warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0)
    {
        const int nw = blockDim.x >> 5;
        int32_t w = lane < nw ? warp_tot[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o)
                w += y;
        }
        if (lane < nw)
            warp_tot[lane] = w; // inclusive over warps
    }
    __syncthreads();
    total = warp_tot[(blockDim.x >> 5) - 1];
    const int32_t before = warp == 0 ? 0 : warp_tot[warp - 1];
    __syncthreads();
    return before + inc - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_local(const int32_t *__restrict__ in, int32_t *__restrict__ out,
                                                             int64_t n, int32_t *__restrict__ tile_sums)
{
    __shared__ int32_t warp_tot[32];
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    int32_t v[kScanPer], s = 0;
#pragma unroll
    for (int u = 0; u < kScanPer; ++u)
    {
        v[u] = base + u < n ? in[base + u] : 0;
        s += v[u];
    }
    int32_t total;
    int32_t run = block_exclusive_scan(s, warp_tot, total);
#pragma unroll
    for (int u = 0; u < kScanPer; ++u)
    {
        if (base + u < n)
            out[base + u] = run;
        run += v[u];
    }
    if (threadIdx.x == 0)
        tile_sums[blockIdx.x] = total;
}

// exclusive scan of the tile totals in place (one block, a tile at a time)
__global__ void __launch_bounds__(kScanThreads) k_scan_top(int32_t *__restrict__ sums, int64_t n)
{
    __shared__ int32_t warp_tot[32];
    int32_t carry = 0;
    for (int64_t b0 = 0; b0 < n; b0 += kScanThreads)
    {
        const int64_t i = b0 + threadIdx.x;
        const int32_t v = i < n ? sums[i] : 0;
        int32_t total;
        const int32_t ex = block_exclusive_scan(v, warp_tot, total);
        if (i < n)
            sums[i] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(int32_t *__restrict__ out, int64_t n,
                                                           const int32_t *__restrict__ tile_sums)
{
    const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
    const int32_t add = tile_sums[blockIdx.x];
#pragma unroll
    for (int u = 0; u < kScanPer; ++u)
        if (base + u < n)
            out[base + u] += add;
}

int64_t scan_tiles(int64_t n)
{
    return (n + kScanTile - 1) / kScanTile;
}

cudaError_t exclusive_scan(const int32_t *in, int32_t *out, int64_t n, int32_t *tile_sums, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    const int64_t nt = scan_tiles(n);
    k_scan_local<<<(unsigned)nt, kScanThreads, 0, st>>>(in, out, n, tile_sums);
    cudaError_t e;
    if ((e = launched()))
        return e;
    k_scan_top<<<1, kScanThreads, 0, st>>>(tile_sums, nt);
    if ((e = launched()))
        return e;
    k_scan_add<<<(unsigned)nt, kScanThreads, 0, st>>>(out, n, tile_sums);
    return launched();
}

// ------------------------------------------------------------ product keys
struct ProdOps
{
    const uint64_t *xa, *za, *xb, *zb; // masks in caller order
    int64_t Pb;
    int n;
};

__device__ __forceinline__ void pair_key(const ProdOps &o, int32_t p, uint64_t &x, uint64_t &z)
{
    const int64_t i = (int64_t)p / o.Pb, j = (int64_t)p - i * o.Pb;
    x = o.xa[i] ^ o.xb[j];
    z = o.za[i] ^ o.zb[j];
}

// bits [pos, pos + 4) of the 2n-bit key (x : z), z in the low n bits
__device__ __forceinline__ uint32_t key_digit(uint64_t x, uint64_t z, int n, int pos)
{
    uint32_t d = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t)
    {
        const int b = pos + t;
        const uint64_t bit = b < n ? (z >> b) & 1ull : (b < 2 * n ? (x >> (b - n)) & 1ull : 0ull);
        d |= (uint32_t)bit << t;
    }
    return d;
}

// caller-order masks from the sorted encoding
__global__ void k_prod_masks(const StringRec *__restrict__ recs, const int32_t *__restrict__ orig, int64_t P,
                             uint64_t *__restrict__ xs, uint64_t *__restrict__ zs)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s < P)
    {
        xs[orig[s]] = recs[s].x;
        zs[orig[s]] = recs[s].z;
    }
}

__global__ void k_prod_iota(int32_t *__restrict__ idx, int64_t N)
{
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N; p += (int64_t)gridDim.x * blockDim.x)
        idx[p] = (int32_t)p;
}

// per block: counts of each digit among its kRsTile items -> hist[d * nb + b]
__global__ void __launch_bounds__(kRsThreads) k_rs_hist(const int32_t *__restrict__ idx, int64_t N, ProdOps o, int pos,
                                                        int32_t *__restrict__ hist)
{
    __shared__ int32_t cnt[16];
    if (threadIdx.x < 16)
        cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * kRsTile;
    for (int r = 0; r < kRsRounds; ++r)
    {
        const int64_t q = base + (int64_t)r * kRsThreads + threadIdx.x;
        if (q < N)
        {
            uint64_t x, z;
            pair_key(o, idx[q], x, z);
            atomicAdd(&cnt[key_digit(x, z, o.n, pos)], 1);
        }
    }
    __syncthreads();
    if (threadIdx.x < 16)
        hist[(int64_t)threadIdx.x * gridDim.x + blockIdx.x] = cnt[threadIdx.x];
}

// stable scatter: item q of block b goes to offs[d * nb + b] + (items of
// digit d before it in the block)
__global__ void __launch_bounds__(kRsThreads) k_rs_scatter(const int32_t *__restrict__ idx_in, int32_t *__restrict__ idx_out,
                                                           int64_t N, ProdOps o, int pos,
                                                           const int32_t *__restrict__ offs)
{
    constexpr int NW = kRsThreads / 32;
    __shared__ int32_t running[16];
    __shared__ int32_t wcnt[NW][17];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x < 16)
        running[threadIdx.x] = offs[(int64_t)threadIdx.x * gridDim.x + blockIdx.x];
    const int64_t base = (int64_t)blockIdx.x * kRsTile;
    for (int r = 0; r < kRsRounds; ++r)
    {
        for (int t = threadIdx.x; t < NW * 17; t += kRsThreads)
            wcnt[t / 17][t % 17] = 0;
        __syncthreads();
        const int64_t q = base + (int64_t)r * kRsThreads + threadIdx.x;
        int32_t v = 0;
        uint32_t d = 16; // no item
        if (q < N)
        {
            v = idx_in[q];
            uint64_t x, z;
            pair_key(o, v, x, z);
            d = key_digit(x, z, o.n, pos);
        }
        const uint32_t peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & ((1u << lane) - 1u));
        if (rank == 0)
            wcnt[warp][d] = __popc(peers);
        __syncthreads();
        if (d < 16)
        {
            int32_t before = running[d];
            for (int w = 0; w < warp; ++w)
                before += wcnt[w][d];
            idx_out[before + rank] = v;
        }
        __syncthreads();
        if (threadIdx.x < 16)
        {
            int32_t add = 0;
            for (int w = 0; w < NW; ++w)
                add += wcnt[w][threadIdx.x];
            running[threadIdx.x] += add;
        }
        __syncthreads();
    }
}

// flags[q] = 1 where a run of equal keys starts
__global__ void k_prod_heads(const int32_t *__restrict__ idx, int64_t N, ProdOps o, int32_t *__restrict__ flags)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x)
    {
        uint64_t x, z;
        pair_key(o, idx[q], x, z);
        int32_t f = 1;
        if (q > 0)
        {
            uint64_t x0, z0;
            pair_key(o, idx[q - 1], x0, z0);
            f = (x != x0 || z != z0) ? 1 : 0;
        }
        flags[q] = f;
    }
}

// one thread per run: sum of i^e a_i b_j over the run, in pair order
__global__ void k_prod_reduce(const int32_t *__restrict__ idx, const int32_t *__restrict__ flags,
                              const int32_t *__restrict__ pos, int64_t N, ProdOps o, const double2 *__restrict__ ca,
                              const double2 *__restrict__ cb, uint64_t *__restrict__ out_x,
                              uint64_t *__restrict__ out_z, double2 *__restrict__ out_c)
{
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < N; q += (int64_t)gridDim.x * blockDim.x)
    {
        if (!flags[q])
            continue;
        double re = 0.0, im = 0.0;
        uint64_t x = 0, z = 0;
        int64_t r = q;
        do
        {
            const int32_t p = idx[r];
            const int64_t i = (int64_t)p / o.Pb, j = (int64_t)p - i * o.Pb;
            const uint64_t xi = o.xa[i], zi = o.za[i], xj = o.xb[j], zj = o.zb[j];
            x = xi ^ xj;
            z = zi ^ zj;
            const int e = (__popcll(xi & zi) + __popcll(xj & zj) - __popcll(x & z) + 2 * __popcll(zi & xj)) & 3;
            const double2 a = ca[i], b = cb[j];
            // a b, then times i^e
            const double pr = a.x * b.x - a.y * b.y, pi = a.x * b.y + a.y * b.x;
            switch (e)
            {
            case 0: re += pr; im += pi; break;
            case 1: re -= pi; im += pr; break;
            case 2: re -= pr; im -= pi; break;
            default: re += pi; im -= pr; break;
            }
            ++r;
        } while (r < N && !flags[r]);
        const int32_t k = pos[q];
        out_x[k] = x;
        out_z[k] = z;
        out_c[k] = make_double2(re, im);
    }
}

unsigned grid_of(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * 32;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

size_t al256(size_t b)
{
    return (b + 255) & ~(size_t)255;
}

} // namespace

size_t product_workspace_bytes(int64_t Pa, int64_t Pb)
{
    const int64_t N = Pa * Pb, nb = (N + kRsTile - 1) / kRsTile;
    const int64_t hist = 16 * nb;
    const int64_t tiles = scan_tiles(N > hist ? N : hist);
    return al256((size_t)(Pa + Pb) * 16) + 4 * al256((size_t)N * 4) + 2 * al256((size_t)hist * 4) +
           al256((size_t)tiles * 4) + 256;
}

cudaError_t launch_op_product(const DevOp &a, const void *coeffs_a, const DevOp &b, const void *coeffs_b, int n,
                              void *ws, uint64_t *out_x, uint64_t *out_z, void *out_c, int64_t *n_out,
                              cudaStream_t st)
{
    const int64_t Pa = a.P, Pb = b.P, N = Pa * Pb;
    *n_out = 0;
    if (N <= 0)
        return cudaSuccess;
    const int64_t nb = (N + kRsTile - 1) / kRsTile, hist_n = 16 * nb;
    unsigned char *p = (unsigned char *)(((uintptr_t)ws + 255) & ~(uintptr_t)255);
    uint64_t *xa = (uint64_t *)p, *za = xa + Pa, *xb = za + Pa, *zb = xb + Pb;
    p += al256((size_t)(Pa + Pb) * 16);
    int32_t *idx0 = (int32_t *)p;
    p += al256((size_t)N * 4);
    int32_t *idx1 = (int32_t *)p;
    p += al256((size_t)N * 4);
    int32_t *flags = (int32_t *)p;
    p += al256((size_t)N * 4);
    int32_t *pos = (int32_t *)p;
    p += al256((size_t)N * 4);
    int32_t *hist = (int32_t *)p;
    p += al256((size_t)hist_n * 4);
    int32_t *offs = (int32_t *)p;
    p += al256((size_t)hist_n * 4);
    int32_t *tile_sums = (int32_t *)p;

    cudaError_t e;
    k_prod_masks<<<grid_of(Pa, 256), 256, 0, st>>>(a.recs, a.orig, Pa, xa, za);
    if ((e = launched()))
        return e;
    k_prod_masks<<<grid_of(Pb, 256), 256, 0, st>>>(b.recs, b.orig, Pb, xb, zb);
    if ((e = launched()))
        return e;
    k_prod_iota<<<grid_of(N, 256), 256, 0, st>>>(idx0, N);
    if ((e = launched()))
        return e;
    const ProdOps o{xa, za, xb, zb, Pb, n};
    for (int pos_bit = 0; pos_bit < 2 * n; pos_bit += 4)
    {
        k_rs_hist<<<(unsigned)nb, kRsThreads, 0, st>>>(idx0, N, o, pos_bit, hist);
        if ((e = launched()))
            return e;
        if ((e = exclusive_scan(hist, offs, hist_n, tile_sums, st)))
            return e;
        k_rs_scatter<<<(unsigned)nb, kRsThreads, 0, st>>>(idx0, idx1, N, o, pos_bit, offs);
        if ((e = launched()))
            return e;
        int32_t *t = idx0;
        idx0 = idx1;
        idx1 = t;
    }
    k_prod_heads<<<grid_of(N, 256), 256, 0, st>>>(idx0, N, o, flags);
    if ((e = launched()))
        return e;
    if ((e = exclusive_scan(flags, pos, N, tile_sums, st)))
        return e;
    k_prod_reduce<<<grid_of(N, 256), 256, 0, st>>>(idx0, flags, pos, N, o, (const double2 *)coeffs_a,
                                                   (const double2 *)coeffs_b, out_x, out_z, (double2 *)out_c);
    if ((e = launched()))
        return e;
    int32_t last[2];
    if ((e = cudaMemcpyAsync(&last[0], pos + N - 1, 4, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaMemcpyAsync(&last[1], flags + N - 1, 4, cudaMemcpyDeviceToHost, st)) ||
        (e = cudaStreamSynchronize(st)))
        return e;
    *n_out = (int64_t)last[0] + last[1];
    return cudaSuccess;
}

} // namespace fpg
