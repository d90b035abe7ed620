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
