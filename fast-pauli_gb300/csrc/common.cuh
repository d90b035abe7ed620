// common.cuh -- shared declarations of the GB300 Pauli engine (internal).
//
// Encoding.  Pauli string character q (0 = leftmost) acts on row-index bit
// (n-1-q).  A string is (x, z, nY) with
//   x = bits of X and Y factors, z = bits of Y and Z factors, nY = #Y,
// so that its matrix has exactly one non-zero per row:
//   column(i) = i ^ x,   value(i) = (-i)^nY * (-1)^popcount(i & z).
// This is the closed form of the reference's get_sparse_repr
// (fast_pauli/cpp/include/__pauli_string.hpp:49-118).
//
// Strings are sorted by x ("x-groups"): every string of a group pairs row i
// with the same row i ^ x, so one load of the row pair serves the whole group.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace fpg
{

// One Pauli string in sorted (x, parity of nY, z) order; 24 bytes.
struct StringRec
{
    uint64_t x;
    uint64_t z;
    uint32_t mask_lo; // bit r (r < 32) = parity(popcount(r & z & 31))
    uint32_t meta;    // bits 0..1: nY mod 4; bits 8..31 unused
};

// Original (caller-order) index of each sorted string is kept separately.

// Work unit of the expectation kernel: up to a class maximum of strings of one
// x-group, n_even strings with even nY at sorted positions
// [begin_even, begin_even + n_even) and n_odd strings with odd nY at
// [begin_odd, begin_odd + n_odd).
struct Chunk
{
    uint64_t x;
    int32_t begin_even;
    int32_t begin_odd;
    int16_t n_even;
    int16_t n_odd;
    int32_t pad;
};

struct Group
{
    uint64_t x;
    int32_t begin;
    int32_t count;
};

// Work unit of the transform kernel (k_expect_wht.cu): `count` consecutive
// sorted strings of one x-group starting at `begin`, the first n_even with
// even #Y.  Groups with at least kWhtMinStrings strings use it, in pieces of
// at most kWhtMaxStrings.
struct WhtChunk
{
    uint64_t x;
    int32_t begin;
    int16_t count;
    int16_t n_even;
};
constexpr int kWhtMinStrings = 10;
constexpr int kWhtMaxStrings = 128;
constexpr int kWhtThreads = 256; // CTA of the transform kernel

// Work unit of the pair kernel (k_expect_pair.cu): a whole x-group of at most
// kPairMaxStrings strings [begin, begin + count) whose signs, after dropping
// the pairing bit (top bit of x), use at most row bit `abit` (-1: none).
struct PairChunk
{
    uint64_t x;
    int32_t begin;
    int32_t count;
    int32_t abit;
    int32_t pad;
};
constexpr int kPairMaxStrings = 16;

// Work unit of the tile kernel (k_expect_tile.cu): four row bits
// q[0] < q[1] < q[2] < q[3] and up to kTileSlots two-position x-groups
// x = 2^q[i] + 2^q[j], slot s <-> (i, j) = (0,1) (0,2) (1,2) (0,3) (1,3) (2,3),
// whose strings [begin[s], begin[s] + count[s]) all have z' in {0, 2^q[i]}
// (count 0: empty slot).
constexpr int kTileSlots = 6;
struct TileChunk
{
    int32_t begin[kTileSlots];
    int8_t count[kTileSlots];
    int8_t q[4];
    int8_t pad[6];
};

// Work unit of the marginal kernel (k_expect_marg.cu): a whole x-group
// [begin, begin + count) whose strings each have z' (z without the pairing
// bit) of at most one bit; zmask = the union of the z', of which at most
// kMargMaxHighBits bits lie at row bit 5 or above.  flags: bit 0 = the
// group has strings with even #Y (needs Re q), bit 1 = odd #Y (Im q).
struct MargChunk
{
    uint64_t x;
    uint64_t zmask;
    int32_t begin;
    int32_t count;
    int32_t flags;
    int32_t pad;
};
constexpr int kMargMaxHighBits = 18;
constexpr int kMargMinStrings = 4;

// Device-side view of an encoded operator.
struct DevOp
{
    int n;
    int64_t P;
    int64_t G;
    const StringRec *recs; // [P] sorted
    const int32_t *orig;   // [P] sorted position -> caller index
    const Group *groups;   // [G]
};

// ---------------------------------------------------------------------------
// launchers (implemented in k_*.cu); each enqueues one kernel on `st` and
// returns launched(): the launch's cudaError_t, after counting the launch
// (fpg_kernel_launches reports the running total).
// ---------------------------------------------------------------------------
cudaError_t launched();

// Multiprocessor count of the current device (cached per device ordinal;
// 152 on a GB300).  Grid sizes are multiples of it.
int sm_count();

// Chunk classes of the expectation kernel: (max even strings, max odd strings).
constexpr int kNumChunkClasses = 8;
struct ChunkClass
{
    int ge, go;
};
extern const ChunkClass kChunkClasses[kNumChunkClasses];
int chunk_class_for(int n_even, int n_odd); // smallest class covering, -1 if none

// Column tiling for L2 residency.  All chunks of a launch sweep the same
// column tile (2^n rows x TC lanes x bytes per lane) before moving to the
// next, so the state is read from DRAM about once per launch when the tile
// fits in the 126 MB L2.  L2 holds whole 128-byte lines, so a tile narrower
// than 128 bytes per row costs as much L2 as a 128-byte one: narrow the tile
// (halve TC) until it fits the budget, but not below one line per row.
constexpr int64_t kColumnTileBytes = int64_t(40) << 20;
constexpr int kL2Line = 128;
inline int column_lanes_for_l2(int tc, int n, int bytes_per_lane, int64_t budget)
{
    const int min_tc = bytes_per_lane >= kL2Line ? 1 : kL2Line / bytes_per_lane;
    while (tc > min_tc && (int64_t(1) << n) * (int64_t)tc * bytes_per_lane > budget)
        tc >>= 1;
    return tc;
}
// L2 footprint of a column tile (whole lines).
inline int64_t column_tile_footprint(int tc, int n, int bytes_per_lane)
{
    const int64_t w = (int64_t)tc * bytes_per_lane;
    return (int64_t(1) << n) * (w < kL2Line ? kL2Line : w);
}
// When even a one-line tile does not fit, the row range is split so that the
// CTAs running at the same time (chunks fastest, then splits) read rows from
// a window of at most this many 32-row blocks, which L2 can hold.
constexpr int64_t kWindowBlocks = 1024;

// Kernel families of the per-call decomposition; each picks its own row
// splits so that every launch fills the GPU.
enum
{
    kFamDirect = 0,
    kFamPair = 1,
    kFamMarg = 2,
    kFamWht = 3,
    kFamTile = 4,
    kNumFam = 5
};

struct ExpectPlan
{
    int TC;           // column lanes per CTA (power of two <= 32)
    int V;            // complex elements per lane (1 or 2)
    int n_ctiles;     // column tiles
    int n_splits;     // row splits of a launch (>1 -> partial buffer + reduction)
    int wht_TC;       // column lanes of the V = 1 kernels (transform, marginal)
    int wht_ctiles;   // their column tiles
    int fam_splits[kNumFam]; // per-call path: row splits of each family
    bool tile_kernel; // the tile family runs the tile kernel (else the pair kernel)
    int tile_TC;      // its column lanes (one element each) and column tiles
    int tile_ctiles;
};

// ev_or_partial: [n_splits][P][S] float64 (row-major), string index orig[s].
// One launch per class.
cudaError_t launch_expect_chunks(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const Chunk *d_chunks,
                                 int n_chunks, int cls, const ExpectPlan &plan, double *ev_or_partial,
                                 cudaStream_t st);
// ev[glob[l] * S + t] = sum_p partial[(p * Pf + l) * S + t]: the partial table
// of one kernel family (Pf strings in family-local order) into the caller-
// ordered table.
cudaError_t launch_reduce_family(const double *partial, int n_splits, int64_t Pf, int64_t S, const int32_t *glob,
                                 double *ev, cudaStream_t st);

// Pair kernel over pair chunks; uses plan.TC / V / n_ctiles / n_splits like the
// direct kernel and writes like it.  complex128 states run in df64 on the
// float32 pipes (df64.cuh) followed by the float64 form, which recomputes
// only when *range_flag (a device int, zero before the call) was raised;
// psi_df = the state split by launch_df_split (which raises the flag), or
// null to split inside the kernel (which raises it).  complex64 states
// ignore range_flag and psi_df.
cudaError_t launch_expect_pair(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const PairChunk *d_chunks,
                               int n_chunks, const ExpectPlan &plan, double *out, int *range_flag,
                               const void *psi_df, cudaStream_t st);

// Tile kernel over tile units (one complex element per lane, TC column lanes,
// n_ctiles column tiles, 256 threads, n_splits row splits of the 2^(n-4)
// tiles); writes like the pair kernel.  float64: psi = the df64 split copy of
// the state (launch_df_split); values outside the df64 range are left to the
// pair kernel's float64 form (launch_expect_pair_f64_if).  n >= 4.
cudaError_t launch_expect_tile(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const TileChunk *d_units,
                               int n_units, int TC, int n_ctiles, int n_splits, double *out, cudaStream_t st);
// The pair kernel's float64 form alone: returns at once unless *range_flag.
cudaError_t launch_expect_pair_f64_if(const void *psi, int64_t S, int n, const DevOp &op, const PairChunk *d_chunks,
                                      int n_chunks, const ExpectPlan &plan, double *out, const int *range_flag,
                                      cudaStream_t st);

// Marginal kernel over marginal chunks: one complex element per lane, TC
// column lanes (the V = 1 tiling, plan.wht_TC / wht_ctiles), 256 threads;
// max_high_bits = the largest number of zmask bits >= 5 over the chunks.
// range_flag and psi_df as launch_expect_pair.
cudaError_t launch_expect_marg(bool fp32, const void *psi, int64_t S, int n, const DevOp &op,
                               const MargChunk *d_chunks, int n_chunks, int max_high_bits, int TC, int n_ctiles,
                               int n_splits, double *out, int *range_flag, const void *psi_df, cudaStream_t st);

// out[i] = complex128 psi[i] as df64 (re_h, re_l, im_h, im_l) floats for the
// rows x cols row-major elements (out null: the range check only); raises
// *range_flag for elements or columns outside the df64 range (df64.cuh).
// colmax: df_split_colmax_bytes(cols) of scratch.
cudaError_t launch_df_split(const void *psi, int64_t rows, int64_t cols, void *out, void *colmax, int *range_flag,
                            cudaStream_t st);
size_t df_split_colmax_bytes(int64_t cols);
// State size up to which the float64 path splits the state into a scratch
// copy once per call instead of inside every kernel.
constexpr int64_t kDfSplitMaxBytes = int64_t(16) << 30;

// Transform kernel over WHT chunks (kWhtThreads = TC column lanes x
// kWhtThreads/TC row lanes, one complex element per lane); writes like
// launch_expect_chunks.
// complex128: df64 on psi_df then the float64 recomputation gated by
// *range_flag, or float64 alone when psi_df is null.
// both_parts: some chunk has strings of both #Y parities.
cudaError_t launch_expect_wht(bool fp32, const void *psi, int64_t S, int n, const DevOp &op, const WhtChunk *d_chunks,
                              int n_chunks, int max_count, bool both_parts, int TC, int n_ctiles, int n_splits,
                              double *out, int *range_flag, const void *psi_df, cudaStream_t st);

// out(K,S) += H^T(K,P) * E(P,S); H complex (P,K), E real float64 (P,S),
// float64 arithmetic on the CUDA cores (the allocation-free entry point's
// contraction).  out complex128 or complex64 (out_c64).
cudaError_t launch_contract_real(bool out_c64, const void *H, bool h_c64, const double *E, int64_t P, int64_t K,
                                 int64_t S, void *out, cudaStream_t st);

// Tensor-core (tcgen05, 3xTF32, float32 accumulation) forms for the mixed
// path; ws must hold tc_workspace_bytes(M, N, Kd) of the GEMM they run:
//   expectation: M = 2K, N = S, Kd = P;   weighted: M = 2P, N = S, Kd = K.
size_t tc_workspace_bytes(int64_t M, int64_t N, int64_t Kd);
// out(K,S) complex64 += H^T E with H complex64 (P,K), E float64 (P,S)
cudaError_t launch_contract_tc_expect(const void *H, const double *E, int64_t P, int64_t K, int64_t S, void *out,
                                      void *ws, cudaStream_t st);
// W(P,S) complex64 = H X with H complex64 (P,K), X float32 (K,S)
cudaError_t launch_weighted_tc(const void *H, const float *X, int64_t P, int64_t K, int64_t S, void *W, void *ws,
                               cudaStream_t st);
// Float64 form on the tensor cores (bf16 digit slices, exact float32
// accumulation; k_contract_tc.cu): out(K,S) complex128 += H^T E with H
// complex128 (P,K), E float64 (P,S); ws holds oz_workspace_bytes(2K, S, P).
// flag: device int, zero before the call; raised when H or E holds a
// non-finite value, in which case these kernels leave out untouched and
// launch_contract_f64_if computes the contraction.
// The H half of its preparation (row scales and digit slices of H), which
// may run on another stream before the rest (ordered after it by the caller).
size_t oz_workspace_bytes(int64_t M, int64_t N, int64_t Kd);
cudaError_t launch_contract_oz_prep_h(const void *H, int64_t P, int64_t K, int64_t S, void *ws, int *flag,
                                      cudaStream_t st);
cudaError_t launch_contract_oz_expect(const void *H, const double *E, int64_t P, int64_t K, int64_t S, void *out,
                                      void *ws, int *flag, cudaStream_t st);
// The float64 CUDA-core contraction (complex128 H and out), run only when
// *only_if != 0.
cudaError_t launch_contract_f64_if(const void *H, const double *E, int64_t P, int64_t K, int64_t S, void *out,
                                   const int *only_if, cudaStream_t st);
// Reads and clears the tensor-core kernels' device error flag (synchronises st).
cudaError_t read_device_error(int *code, cudaStream_t st);

// W(P,S) complex = H(P,K) complex * X(K,S) real.  Overwrites W.  Precision by fp32.
cudaError_t launch_weighted_coeffs(bool fp32, const void *H, const void *X, int64_t P, int64_t K, int64_t S, void *W,
                                   cudaStream_t st);

// cw_sorted[s] = coeffs[orig[s]] * (-i)^nY   (complex, dtype of coeffs), coeffs: [P] or
// row sums of (P,K) when K > 0.
cudaError_t launch_prep_coeffs(bool fp32, const DevOp &op, const void *coeffs, int64_t K, void *cw_sorted,
                               cudaStream_t st);

// out(D,S) += sum_g psi[i^x_g] * sum_{j in g} cw[j] * (-1)^popc(i & z_j).
// weighted: cw is (P_sorted, S) complex per column (already * phase, sorted order).
// diag (float32, not weighted): the group diagonals from launch_group_diag.
cudaError_t launch_apply(bool fp32, bool weighted, const DevOp &op, const void *cw, const void *psi, void *out,
                         int64_t S, cudaStream_t st, const int *only_if = nullptr, const void *diag = nullptr);
// The float64 apply in df64: cw_df / psi_df are the df64 copies (float4 per
// complex value, launch_df_split) of cw and psi; returns at once when
// *skip_if is set (launch_apply with only_if = skip_if then runs).  diag (not
// weighted): the df64 group diagonals from launch_group_diag.
cudaError_t launch_apply_df(bool weighted, const DevOp &op, const void *cw_df, const void *psi_df, void *out,
                            int64_t S, const int *skip_if, cudaStream_t st, const void *diag = nullptr);
// The group diagonals of a plain apply, diag[g * 2^n + i] = (D_g)_ii for
// every x-group g and row i, from the sorted-order coefficients cw (P values,
// already times the phase): float2 per entry from float32 cw, or (df) float4
// df64 per entry from cw's df64 copy.  Returns at once when skip_if is set.
cudaError_t launch_group_diag(bool df, const DevOp &op, const void *cw, void *diag, const int *skip_if,
                              cudaStream_t st);

// W(P,S) in caller order -> sorted order with phase: cw[s,t] = W[orig[s],t] * (-i)^nY
cudaError_t launch_prep_weighted(bool fp32, const DevOp &op, const void *W, int64_t S, void *cw_sorted,
                                 cudaStream_t st);

// SummedPauliOp::square (k_square.cu): pair lists of the squared strings sq,
// then out(A,K) (overwritten) from h (P,K); ws holds
// square_workspace_bytes(P, A); *found -> device counter of the (i,j) pairs
// whose product was found in sq (P^2 when every product is there).
int64_t square_max_terms(int64_t P);
size_t square_workspace_bytes(int64_t P, int64_t A);
cudaError_t launch_square(bool fp32, const DevOp &op, const DevOp &sq, const void *h, int64_t K, void *out,
                          void *ws, unsigned long long **found, cudaStream_t st);

// PauliOp product with equal strings merged (k_product.cu): the distinct
// strings among the products of a's and b's strings as (x, z) masks sorted
// by (x, z), and their complex128 coefficients; out arrays hold a.P * b.P
// entries (< 2^31), *n_out (host) the count; ws holds
// product_workspace_bytes(a.P, b.P).  Synchronises st.
size_t product_workspace_bytes(int64_t Pa, int64_t Pb);
cudaError_t launch_op_product(const DevOp &a, const void *coeffs_a, const DevOp &b, const void *coeffs_b, int n,
                              void *ws, uint64_t *out_x, uint64_t *out_z, void *out_c, int64_t *n_out,
                              cudaStream_t st);

// out(k, i, j) += (sum_j coeffs(j,k) P_j)(i, j): the dense matrices of K
// operators, out (K, 2^n, 2^n) complex.
cudaError_t launch_to_tensor(bool fp32, const DevOp &op, const void *coeffs, int64_t K, void *out, cudaStream_t st);

cudaError_t launch_sparse_repr(uint64_t x, uint64_t z, int ny, int n, uint64_t *cols, void *vals, cudaStream_t st);

} // namespace fpg
