// host_internal.hpp -- host-side helpers shared by the C-ABI translation units.
#pragma once

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"

namespace fpg
{

// Record msg as the calling thread's last error; returns code.
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *where);

// Encode P strings of n characters ('I','X','Y','Z'): sorted records, the
// sorted->caller index map, x-groups and expectation chunks bucketed by
// kernel class (class c owns chunks [class_begin[c], class_begin[c+1])).
int encode_strings(const char *strings, int64_t P, int n, std::vector<StringRec> &recs, std::vector<int32_t> &orig,
                   std::vector<Group> &groups, std::vector<Chunk> &chunks, std::vector<int> &class_begin);

} // namespace fpg

struct fpg_operator;

namespace fpg
{
// Upper bound of the scratch bytes one expectation (weighted = false) or
// apply_weighted (weighted = true) call draws from the stream-ordered pool.
size_t request_scratch_bytes(const fpg_operator *op, int64_t K, int64_t S, bool fp32, bool weighted);

// One expectation problem of a merged run: out(K,S) = sum_j coeffs(j,k)
// <psi_t|P_j|psi_t> (overwritten), device arrays of the run's dtype.
struct MergedExpect
{
    const fpg_operator *op;
    const void *coeffs;
    int64_t n_operators;
    const void *states;
    void *out;
    int64_t n_states;
};
// Problems run as one batch on `st` without synchronising (batch.cu); each
// problem's result is independent of the others in the run.
int run_merged_expect(int32_t dtype, const MergedExpect *probs, int n, cudaStream_t st);
// Pool bytes one problem adds to a merged run (upper bound for admission).
size_t merged_expect_scratch_bytes(const fpg_operator *op, int64_t S, const void *states, bool fp32);
} // namespace fpg

// An encoded operator: host copies of the encoding and their device mirrors.
struct fpg_operator
{
    int n = 0;
    int64_t P = 0;
    int device = 0;
    std::vector<fpg::StringRec> recs;
    std::vector<int32_t> orig;
    std::vector<fpg::Group> groups;
    std::vector<fpg::Chunk> chunks;
    std::vector<int> class_begin; // chunks of class c: [class_begin[c], class_begin[c+1])
    // per-call decomposition: groups of >= kWhtMinStrings strings go to the
    // transform kernel (wht), the rest to the direct classes (fast_chunks)
    std::vector<fpg::Chunk> fast_chunks;
    std::vector<int> fast_class_begin;
    std::vector<fpg::WhtChunk> wht;
    int wht_max_count = 0;
    bool wht_both = false; // some transform chunk has strings of both #Y parities
    std::vector<fpg::PairChunk> pairs; // groups served by the pair kernel
    fpg::PairChunk *d_pairs = nullptr;
    // two-position groups served by the tile kernel, and the same groups as
    // pair chunks (for the pair kernel when a call cannot use the tile
    // kernel, and for the float64 recomputation)
    std::vector<fpg::TileChunk> tiles;
    fpg::TileChunk *d_tiles = nullptr;
    std::vector<fpg::PairChunk> tile_pairs;
    fpg::PairChunk *d_tile_pairs = nullptr;
    std::vector<fpg::MargChunk> margs; // groups served by the marginal kernel
    int marg_max_high = 0;
    fpg::MargChunk *d_margs = nullptr;
    // strings by kernel family: local[s] = index of sorted string s within its
    // family; glob[fam_begin[f] + l] = caller index of family f's string l
    std::vector<int32_t> local;
    std::vector<int32_t> glob;
    int64_t fam_begin[fpg::kNumFam + 1] = {};
    int32_t *d_local = nullptr;
    int32_t *d_glob = nullptr;
    fpg::StringRec *d_recs = nullptr;
    int32_t *d_orig = nullptr;
    fpg::Group *d_groups = nullptr;
    fpg::Chunk *d_chunks = nullptr;
    fpg::Chunk *d_fast_chunks = nullptr;
    fpg::WhtChunk *d_wht = nullptr;

    fpg::DevOp dev() const
    {
        return fpg::DevOp{n, P, (int64_t)groups.size(), d_recs, d_orig, d_groups};
    }
};
